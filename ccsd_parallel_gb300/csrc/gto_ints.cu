// Gaussian one- and two-electron integrals on the GPU: the producer of the
// CCSD inputs, replacing the reference's Hartree_Integrals (hartree_integrals.cpp:
// 293-796) and the (mu nu|la si) loop of Hartree_Fock_Solver::get_Energy
// (hartree_fock_solver.cpp:714-817), which run one contracted integral at a time
// on the host.
//
// McMurchie-Davidson over contracted Cartesian Gaussians, as the reference:
//   - a primitive-pair table, one block per basis-function pair i >= j: exponent
//     sum p, centre P, c_k c_m and the Hermite coefficients E_t^{l_i l_j} of each
//     dimension (Fill_E_ij recursion, hartree_integrals.cpp:160-210);
//   - one thread per pair for S, <mu|nabla^2|nu> and sum_C Z_C <mu|1/r_C|nu>;
//   - one thread per unique quartet (ij|kl), (ij) >= (kl), for the ERIs: for each
//     primitive quartet the Boys function (below x = 50 the reference's series for F_30
//     and downward recursion, above it the asymptotic form, :643-693), the
//     Hermite Coulomb integrals R_tuv (Set_R_ijk, :23-94) two levels of n at a time
//     in a local buffer, and the E (-1)^{t'+u'+v'} E R contraction (:720-796); the
//     value lands in its 8 symmetric places.
// FP64 throughout: the outputs feed an FP64 SCF and CCSD.
#include <algorithm>
#include <cmath>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/ccsd_gb300.h"
#include "common.h"

namespace ccsd {
void set_last_error(const std::string &msg);

namespace {

constexpr int kLMax = 3;                  // f functions (the reference's largest tables)
constexpr int kET = 2 * kLMax + 1;        // E_t, t <= l_i + l_j
constexpr int kBoysN = 30;                // the reference's top order

struct PrimPair {
    double p, P[3], K;        // exponent sum, centre, c_k c_m
    double E[3][kET];         // E_t^{l_i l_j} per dimension (with its exp factor)
};

__constant__ double c_inv_series[100];    // 1 / (2 kBoysN + 1 + 2 j)
__constant__ double c_inv_odd[kBoysN + 1];  // 1 / (2 i - 1)
__constant__ double c_boys_start;         // (2 kBoysN - 1)!! / 2^(kBoysN + 1), as Set_Boys_Start

// F_m(x_k) for x_k = k h, k <= kTabN - 1 (x <= 50), m < kTabM, from the series below
constexpr int kTabN = 1001, kTabM = 4 * kLMax + 7;
constexpr double kTabH = 0.05;
__constant__ const double *c_boys_tab;

__device__ __forceinline__ int tri_row(long long q) {
    // largest r with r (r + 1) / 2 <= q
    long long r = (long long)((sqrt(8.0 * (double)q + 1.0) - 1.0) * 0.5);
    while (r * (r + 1) / 2 > q) --r;
    while ((r + 1) * (r + 2) / 2 <= q) ++r;
    return (int)r;
}

// F_0 .. F_nmax at x (nmax <= kBoysN), the reference's way (Boys,
// hartree_integrals.cpp:643-693): F_30 from its series below x = 50, from the
// asymptotic form (59)!!/2^31 sqrt(pi/x^61) above, then F_{i-1} = (2x F_i + e^{-x}) /
// (2i - 1) down to F_0.  That asymptotic form needs x >> 30: just above 50 it is off
// by 1.2e-3 (relative), 1e-5 at 60, 1e-11 at 80, and x^61 overflows to F = 0 above
// x = 1.1e5.  accurate = true takes x > 50 from F_0 = sqrt(pi/x)/2 upward instead
// (F_{n+1} = (2n+1)/(2x) F_n, accurate to e^{-x}).
//
// Below x = 50 the values come from a table of the same series on a grid of step
// h = 0.05: F_nmax(x) = sum_{j<7} F_{nmax+j}(x_k) (x_k - x)^j / j! about the nearest
// x_k (truncation below (h/2)^7/7! = 1.2e-15 relative), then the same downward
// recursion.  The table is built once by the series (boys_table_kernel).
__device__ double boys_series30(double x, double ex) {
    double term = c_inv_series[0], sum = term;
    const double tx = 2.0 * x;
    for (int j = 1; j < 100; ++j) {
        term *= tx * c_inv_series[j];
        sum += term;
        if (term < 1e-17 * sum) break;
    }
    return sum * ex;
}

__device__ void boys(int nmax, double x, double *F, bool accurate) {
    if (x > 50.0 && accurate) {
        F[0] = 0.5 * sqrt(M_PI / x);
        const double h = 0.5 / x;
        for (int n = 0; n < nmax; ++n) F[n + 1] = (2 * n + 1) * h * F[n];
        return;
    }
    const double ex = exp(-x);
    if (x <= 50.0 && c_boys_tab && nmax + 6 < kTabM) {
        const int k = (int)(x * (1.0 / kTabH) + 0.5);
        const double d = k * kTabH - x;  // x_k - x
        const double *T = c_boys_tab + (size_t)k * kTabM + nmax;
        double f = T[6];
        f = T[5] + f * d * (1.0 / 6.0);
        f = T[4] + f * d * (1.0 / 5.0);
        f = T[3] + f * d * (1.0 / 4.0);
        f = T[2] + f * d * (1.0 / 3.0);
        f = T[1] + f * d * (1.0 / 2.0);
        f = T[0] + f * d;
        F[nmax] = f;
        for (int i = nmax; i > 0; --i) F[i - 1] = (2.0 * x * F[i] + ex) * c_inv_odd[i];
        return;
    }
    double f;
    if (x > 50.0) {
        f = c_boys_start * sqrt(M_PI / pow(x, 2.0 * kBoysN + 1.0));
    } else {
        f = boys_series30(x, ex);
    }
    for (int i = kBoysN; i > 0; --i) {
        if (i <= nmax) F[i] = f;
        f = (2.0 * x * f + ex) * c_inv_odd[i];
    }
    F[0] = f;
}

// E[i][j][t] for i <= la, j <= lb + 2 (the +2 for the kinetic integrals), one dimension
struct HermiteTable {
    double E[kLMax + 1][kLMax + 3][2 * kLMax + 4];
};

__device__ void hermite_1d(int la, int lbx, double a, double b, double A, double B, HermiteTable &T) {
    const double p = a + b, h = 0.5 / p, P = (a * A + b * B) / p;
    const double XPA = P - A, XPB = P - B, XAB = A - B;
    for (int i = 0; i <= la; ++i)
        for (int j = 0; j <= lbx; ++j)
            for (int t = 0; t < 2 * kLMax + 4; ++t) T.E[i][j][t] = 0.0;
    T.E[0][0][0] = exp(-a * b / p * XAB * XAB);
    for (int i = 0; i < la; ++i)
        for (int t = 0; t <= i + 1; ++t)
            T.E[i + 1][0][t] = (t ? h * T.E[i][0][t - 1] : 0.0) + XPA * T.E[i][0][t] +
                               (t + 1 <= i ? (t + 1) * T.E[i][0][t + 1] : 0.0);
    for (int i = 0; i <= la; ++i)
        for (int j = 0; j < lbx; ++j)
            for (int t = 0; t <= i + j + 1; ++t)
                T.E[i][j + 1][t] = (t ? h * T.E[i][j][t - 1] : 0.0) + XPB * T.E[i][j][t] +
                                   (t + 1 <= i + j ? (t + 1) * T.E[i][j][t + 1] : 0.0);
}

// R^0_{tuv} for t <= T, u <= U, v <= W into R[(t (U+1) + u) (W+1) + v]; two levels of n
// in cur/nxt (each (T+1)(U+1)(W+1) <= RB long)
template <int RB>
__device__ void hermite_R(double alpha, double X, double Y, double Zc, int T, int U, int W, double *R,
                          bool accurate) {
    const int L = T + U + W;
    double F[kBoysN + 1];
    boys(L, alpha * (X * X + Y * Y + Zc * Zc), F, accurate);
    double buf[2][RB];
    const int su = W + 1, st = (U + 1) * su;
    double m2a[kBoysN + 1];  // (-2 alpha)^n
    m2a[0] = 1.0;
    for (int k = 0; k < L; ++k) m2a[k + 1] = m2a[k] * (-2.0 * alpha);
    double *nx = buf[0], *cu = buf[1];  // nx: level n + 1, cu: level n
    nx[0] = m2a[L] * F[L];
    for (int n = L - 1; n >= 0; --n) {
        const int s = L - n;  // entries with t + u + v <= s at level n
        for (int t = 0; t <= T && t <= s; ++t)
            for (int u = 0; u <= U && t + u <= s; ++u)
                for (int v = 0; v <= W && t + u + v <= s; ++v) {
                    double r;
                    if (t == 0 && u == 0 && v == 0) {
                        r = m2a[n] * F[n];
                    } else if (t > 0) {
                        r = X * nx[(t - 1) * st + u * su + v];
                        if (t > 1) r += (t - 1) * nx[(t - 2) * st + u * su + v];
                    } else if (u > 0) {
                        r = Y * nx[(u - 1) * su + v];
                        if (u > 1) r += (u - 1) * nx[(u - 2) * su + v];
                    } else {
                        r = Zc * nx[v - 1];
                        if (v > 1) r += (v - 1) * nx[v - 2];
                    }
                    cu[t * st + u * su + v] = r;
                }
        double *tmp = nx;
        nx = cu;
        cu = tmp;
    }
    for (int i = 0; i < (T + 1) * st; ++i) R[i] = nx[i];
}

__global__ void boys_table_kernel(double *tab) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= kTabN) return;
    const double x = k * kTabH, ex = exp(-x);
    double f = boys_series30(x, ex);
    for (int i = kBoysN; i > 0; --i) {
        if (i < kTabM) tab[(size_t)k * kTabM + i] = f;
        f = (2.0 * x * f + ex) * c_inv_odd[i];
    }
    tab[(size_t)k * kTabM] = f;
}

struct BasisDev {
    const int *atom, *pw, *nprim;
    const double *alpha, *coef, *R, *Z;
    int n, maxprim, natoms;
    bool accurate;  // Boys above x = 50 from F_0's asymptotic form
};

// one block per basis-function pair i >= j; threads over its primitive pairs
__global__ void prim_pair_kernel(BasisDev b, const long long *pp_off, PrimPair *pp) {
    const int P = blockIdx.x;
    const int i = tri_row(P), j = P - i * (i + 1) / 2;
    const int ni = b.nprim[i], nj = b.nprim[j];
    const double *A = b.R + 3 * b.atom[i], *B = b.R + 3 * b.atom[j];
    for (int e = threadIdx.x; e < ni * nj; e += blockDim.x) {
        const int k = e / nj, m = e % nj;
        const double a1 = b.alpha[i * b.maxprim + k], a2 = b.alpha[j * b.maxprim + m];
        PrimPair r;
        r.p = a1 + a2;
        r.K = b.coef[i * b.maxprim + k] * b.coef[j * b.maxprim + m];
        HermiteTable T;
        for (int d = 0; d < 3; ++d) {
            const int li = b.pw[3 * i + d], lj = b.pw[3 * j + d];
            r.P[d] = (a1 * A[d] + a2 * B[d]) / r.p;
            hermite_1d(li, lj, a1, a2, A[d], B[d], T);
            for (int t = 0; t < kET; ++t) r.E[d][t] = t <= li + lj ? T.E[li][lj][t] : 0.0;
        }
        pp[pp_off[P] + e] = r;
    }
}

// S, <mu|nabla^2|nu>, sum_C Z_C <mu|1/r_C|nu> for each pair i >= j (both triangles written)
__global__ void one_electron_kernel(BasisDev b, double *S, double *lap, double *nuc) {
    const int npair = b.n * (b.n + 1) / 2;
    for (int P = blockIdx.x * blockDim.x + threadIdx.x; P < npair; P += gridDim.x * blockDim.x) {
        const int i = tri_row(P), j = P - i * (i + 1) / 2;
        const double *A = b.R + 3 * b.atom[i], *B = b.R + 3 * b.atom[j];
        int li[3], lj[3];
        for (int d = 0; d < 3; ++d) {
            li[d] = b.pw[3 * i + d];
            lj[d] = b.pw[3 * j + d];
        }
        double s = 0.0, k2 = 0.0, vn = 0.0;
        for (int k = 0; k < b.nprim[i]; ++k)
            for (int m = 0; m < b.nprim[j]; ++m) {
                const double a1 = b.alpha[i * b.maxprim + k], a2 = b.alpha[j * b.maxprim + m], p = a1 + a2;
                const double cc = b.coef[i * b.maxprim + k] * b.coef[j * b.maxprim + m];
                double e0[3], ek[3], Et[3][kET], P[3];
                HermiteTable T;
                for (int d = 0; d < 3; ++d) {
                    hermite_1d(li[d], lj[d] + 2, a1, a2, A[d], B[d], T);
                    const int D = lj[d];
                    e0[d] = T.E[li[d]][D][0];
                    ek[d] = 4.0 * a2 * a2 * T.E[li[d]][D + 2][0] - 2.0 * a2 * (2 * D + 1) * T.E[li[d]][D][0];
                    if (D > 1) ek[d] += D * (D - 1) * T.E[li[d]][D - 2][0];
                    for (int t = 0; t < kET; ++t) Et[d][t] = t <= li[d] + D ? T.E[li[d]][D][t] : 0.0;
                    P[d] = (a1 * A[d] + a2 * B[d]) / p;
                }
                const double pre = cc * pow(M_PI / p, 1.5);
                s += pre * e0[0] * e0[1] * e0[2];
                k2 += pre * (ek[0] * e0[1] * e0[2] + e0[0] * ek[1] * e0[2] + e0[0] * e0[1] * ek[2]);
                const int Tx = li[0] + lj[0], Uy = li[1] + lj[1], Wz = li[2] + lj[2];
                double R[64];  // (Tx+1)(Uy+1)(Wz+1) <= 27 for l <= 3 on each function
                double acc = 0.0;
                for (int c = 0; c < b.natoms; ++c) {
                    const double *C = b.R + 3 * c;
                    hermite_R<64>(p, P[0] - C[0], P[1] - C[1], P[2] - C[2], Tx, Uy, Wz, R, b.accurate);
                    double sum = 0.0;
                    for (int t = 0; t <= Tx; ++t)
                        for (int u = 0; u <= Uy; ++u)
                            for (int v = 0; v <= Wz; ++v)
                                sum += Et[0][t] * Et[1][u] * Et[2][v] * R[(t * (Uy + 1) + u) * (Wz + 1) + v];
                    acc += b.Z[c] * sum;
                }
                vn += cc * acc * 2.0 * M_PI / p;
            }
        const size_t ij = (size_t)i * b.n + j, ji = (size_t)j * b.n + i;
        if (S) S[ij] = S[ji] = s;
        if (lap) lap[ij] = lap[ji] = k2;
        if (nuc) nuc[ij] = nuc[ji] = vn;
    }
}

// (ij|kl) for each unique quartet: q enumerates (a >= b) over the function pairs in
// `order` (sorted by angular momentum and primitive count, so that the threads of a
// warp do alike work); RB bounds (Tx+1)(Uy+1)(Wz+1)
template <int RB>
__global__ void __launch_bounds__(128) eri_kernel(int n, long long nquart, const int *pw, const long long *pp_off,
                                                  const PrimPair *pp, const int *order, double *eri, bool accurate) {
    const double pref = 2.0 * pow(M_PI, 2.5);
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < nquart;
         q += (long long)gridDim.x * blockDim.x) {
        const int a = tri_row(q), b = (int)(q - (long long)a * (a + 1) / 2);
        const int P1 = order[a], P2 = order[b];
        const int i = tri_row(P1), j = P1 - i * (i + 1) / 2;
        const int k = tri_row(P2), l = P2 - k * (k + 1) / 2;
        int Lb[3], Lk[3];
        for (int d = 0; d < 3; ++d) {
            Lb[d] = pw[3 * i + d] + pw[3 * j + d];
            Lk[d] = pw[3 * k + d] + pw[3 * l + d];
        }
        const int Tx = Lb[0] + Lk[0], Uy = Lb[1] + Lk[1], Wz = Lb[2] + Lk[2];
        const int su = Wz + 1, st = (Uy + 1) * su;
        double R[RB];
        double val = 0.0;
        for (long long a = pp_off[P1]; a < pp_off[P1 + 1]; ++a) {
            const PrimPair &x = pp[a];
            for (long long c = pp_off[P2]; c < pp_off[P2 + 1]; ++c) {
                const PrimPair &y = pp[c];
                const double p = x.p, qq = y.p, alpha = p * qq / (p + qq);
                hermite_R<RB>(alpha, x.P[0] - y.P[0], x.P[1] - y.P[1], x.P[2] - y.P[2], Tx, Uy, Wz, R, accurate);
                double s = 0.0;
                for (int t = 0; t <= Lb[0]; ++t)
                    for (int u = 0; u <= Lb[1]; ++u)
                        for (int v = 0; v <= Lb[2]; ++v) {
                            const double e1 = x.E[0][t] * x.E[1][u] * x.E[2][v];
                            if (e1 == 0.0) continue;
                            double inner = 0.0;
                            for (int t2 = 0; t2 <= Lk[0]; ++t2)
                                for (int u2 = 0; u2 <= Lk[1]; ++u2)
                                    for (int v2 = 0; v2 <= Lk[2]; ++v2) {
                                        const double e2 = y.E[0][t2] * y.E[1][u2] * y.E[2][v2];
                                        const double r = R[(t + t2) * st + (u + u2) * su + v + v2];
                                        inner += ((t2 + u2 + v2) & 1) ? -e2 * r : e2 * r;
                                    }
                            s += e1 * inner;
                        }
                val += x.K * y.K * s * pref / (p * qq * sqrt(p + qq));
            }
        }
        const size_t N = n;
        const size_t ij = (size_t)i * N + j, ji = (size_t)j * N + i, kl = (size_t)k * N + l, lk = (size_t)l * N + k;
        const size_t NN = N * N;
        eri[ij * NN + kl] = val;
        eri[ji * NN + kl] = val;
        eri[ij * NN + lk] = val;
        eri[ji * NN + lk] = val;
        eri[kl * NN + ij] = val;
        eri[kl * NN + ji] = val;
        eri[lk * NN + ij] = val;
        eri[lk * NN + ji] = val;
    }
}

struct DevBuf {
    void *p = nullptr;
    ~DevBuf() {
        if (p) cudaFree(p);
    }
    template <class T>
    T *alloc(size_t n) {
        CCSD_CUDA(cudaMalloc(&p, n * sizeof(T) + 16));
        return (T *)p;
    }
};

// __constant__ memory and the table belong to the current device: set up once per device
void set_constants() {
    static std::mutex mu;
    static std::vector<bool> done;
    int dev = 0;
    CCSD_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(mu);
    if ((int)done.size() > dev && done[dev]) return;
    double inv_series[100], inv_odd[kBoysN + 1];
    for (int j = 0; j < 100; ++j) inv_series[j] = 1.0 / (2.0 * kBoysN + 1.0 + 2.0 * j);
    inv_odd[0] = 0.0;
    for (int i = 1; i <= kBoysN; ++i) inv_odd[i] = 1.0 / (2.0 * i - 1.0);
    double dfac = 1.0;  // (2N - 1)!!, the loop of Set_Boys_Start (hartree_integrals.cpp:264-280)
    for (double i = 1.0; i < 2.0 * kBoysN - 1.0;) {
        i += 2.0;
        dfac *= i;
    }
    const double start = dfac / std::pow(2.0, kBoysN + 1);
    CCSD_CUDA(cudaMemcpyToSymbol(c_inv_series, inv_series, sizeof inv_series));
    CCSD_CUDA(cudaMemcpyToSymbol(c_inv_odd, inv_odd, sizeof inv_odd));
    CCSD_CUDA(cudaMemcpyToSymbol(c_boys_start, &start, sizeof start));
    // the Boys table, built once per process by the series (it lives as long as the process)
    double *tab = nullptr;
    CCSD_CUDA(cudaMalloc(&tab, sizeof(double) * kTabN * kTabM));
    const double *null_tab = nullptr;
    CCSD_CUDA(cudaMemcpyToSymbol(c_boys_tab, &null_tab, sizeof null_tab));
    boys_table_kernel<<<(kTabN + 127) / 128, 128>>>(tab);
    CCSD_LAUNCH_CHECK();
    CCSD_CUDA(cudaDeviceSynchronize());
    const double *ctab = tab;
    CCSD_CUDA(cudaMemcpyToSymbol(c_boys_tab, &ctab, sizeof ctab));
    if ((int)done.size() <= dev) done.resize(dev + 1, false);
    done[dev] = true;
}

}  // namespace

void ao_integrals(const ccsd_basis &bs, double *S, double *T, double *V, double *eri, double *e_nuc,
                  bool device_out, cudaStream_t st) {
    const int n = bs.nbf, na = bs.natoms, mp = bs.maxprim;
    if (n <= 0 || na <= 0 || mp <= 0 || !bs.Z || !bs.R || !bs.atom || !bs.powers || !bs.nprim || !bs.alpha ||
        !bs.coef)
        throw Error(CCSD_ERR_INVALID_ARG, "ccsd_ao_integrals: empty basis or NULL array");
    long long npp_total = 0;
    std::vector<long long> off((size_t)n * (n + 1) / 2 + 1, 0);
    int lmax = 0;
    for (int i = 0; i < n; ++i) {
        if (bs.atom[i] < 0 || bs.atom[i] >= na || bs.nprim[i] <= 0 || bs.nprim[i] > mp)
            throw Error(CCSD_ERR_INVALID_ARG, "ccsd_ao_integrals: bad atom index or primitive count");
        for (int d = 0; d < 3; ++d) {
            const int l = bs.powers[3 * i + d];
            if (l < 0 || l > kLMax) throw Error(CCSD_ERR_UNSUPPORTED, "ccsd_ao_integrals: Cartesian power above 3");
            lmax = std::max(lmax, l);
        }
        if (bs.powers[3 * i] + bs.powers[3 * i + 1] + bs.powers[3 * i + 2] > kLMax)
            throw Error(CCSD_ERR_UNSUPPORTED, "ccsd_ao_integrals: angular momentum above f");
    }
    for (int i = 0, P = 0; i < n; ++i)
        for (int j = 0; j <= i; ++j, ++P) {
            npp_total += (long long)bs.nprim[i] * bs.nprim[j];
            off[P + 1] = npp_total;
        }
    if (e_nuc) {
        double e = 0.0;
        for (int a = 0; a < na; ++a)
            for (int c = 0; c < a; ++c) {
                const double dx = bs.R[3 * a] - bs.R[3 * c], dy = bs.R[3 * a + 1] - bs.R[3 * c + 1],
                             dz = bs.R[3 * a + 2] - bs.R[3 * c + 2];
                e += bs.Z[a] * bs.Z[c] / std::sqrt(dx * dx + dy * dy + dz * dz);
            }
        *e_nuc = e;
    }
    set_constants();
    DevBuf d_atom, d_pw, d_np, d_al, d_co, d_R, d_Z, d_off, d_pp, d_S, d_L, d_N, d_eri, d_ord;
    int *atom = d_atom.alloc<int>(n), *pw = d_pw.alloc<int>(3 * n), *np_ = d_np.alloc<int>(n);
    double *al = d_al.alloc<double>((size_t)n * mp), *co = d_co.alloc<double>((size_t)n * mp);
    double *R = d_R.alloc<double>(3 * na), *Z = d_Z.alloc<double>(na);
    long long *poff = d_off.alloc<long long>(off.size());
    PrimPair *pp = d_pp.alloc<PrimPair>((size_t)npp_total);
    auto up = [&](void *dst, const void *src, size_t bytes) {
        CCSD_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st));
    };
    up(atom, bs.atom, sizeof(int) * n);
    up(pw, bs.powers, sizeof(int) * 3 * n);
    up(np_, bs.nprim, sizeof(int) * n);
    up(al, bs.alpha, sizeof(double) * n * mp);
    up(co, bs.coef, sizeof(double) * n * mp);
    up(R, bs.R, sizeof(double) * 3 * na);
    up(Z, bs.Z, sizeof(double) * na);
    up(poff, off.data(), sizeof(long long) * off.size());
    const bool accurate = (bs.flags & CCSD_BASIS_ACCURATE_BOYS) != 0;
    BasisDev b{atom, pw, np_, al, co, R, Z, n, mp, na, accurate};
    const int npair = n * (n + 1) / 2;
    prim_pair_kernel<<<npair, 128, 0, st>>>(b, poff, pp);
    CCSD_LAUNCH_CHECK();

    const size_t nn = (size_t)n * n;
    auto out_buf = [&](double *user, DevBuf &tmp, size_t count) -> double * {
        if (!user) return nullptr;
        return device_out ? user : tmp.alloc<double>(count);
    };
    double *dS = out_buf(S, d_S, nn), *dL = out_buf(T, d_L, nn), *dN = out_buf(V, d_N, nn);
    if (dS || dL || dN) {
        // every output of the kernel is written; T and V are formed from lap and nuc below
        double *s_ = dS ? dS : d_S.alloc<double>(nn);
        double *l_ = dL ? dL : d_L.alloc<double>(nn);
        double *v_ = dN ? dN : d_N.alloc<double>(nn);
        one_electron_kernel<<<(npair + 127) / 128, 128, 0, st>>>(b, s_, l_, v_);
        CCSD_LAUNCH_CHECK();
        // T = -1/2 <mu|nabla^2|nu>, V = -sum_C Z_C <mu|1/r_C|nu>
        axpby_view((int)n, (int)n, -0.5, MatView{l_, ix1(n), ix1(1)}, 0.0, OutView{l_, ix1(n), ix1(1)}, st);
        axpby_view((int)n, (int)n, -1.0, MatView{v_, ix1(n), ix1(1)}, 0.0, OutView{v_, ix1(n), ix1(1)}, st);
    }
    if (eri) {
        const long long np = npair, nquart = np * (np + 1) / 2;
        // pairs by (l_i + l_j, primitive pairs): neighbouring quartets then cost alike
        std::vector<int> ord(npair), key(npair);
        for (int i = 0, P = 0; i < n; ++i)
            for (int j = 0; j <= i; ++j, ++P) {
                const int L = bs.powers[3 * i] + bs.powers[3 * i + 1] + bs.powers[3 * i + 2] + bs.powers[3 * j] +
                              bs.powers[3 * j + 1] + bs.powers[3 * j + 2];
                key[P] = L * 100000 + bs.nprim[i] * bs.nprim[j];
                ord[P] = P;
            }
        std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) { return key[x] < key[y]; });
        int *dord = d_ord.alloc<int>(npair);
        up(dord, ord.data(), sizeof(int) * npair);
        double *dE = device_out ? eri : d_eri.alloc<double>(nn * nn);
        const int L = 4 * lmax;
        const int blocks = (int)std::min<long long>((nquart + 127) / 128, 152LL * 64);
        if (L <= 4)
            eri_kernel<12><<<blocks, 128, 0, st>>>(n, nquart, pw, poff, pp, dord, dE, accurate);
        else if (L <= 8)
            eri_kernel<48><<<blocks, 128, 0, st>>>(n, nquart, pw, poff, pp, dord, dE, accurate);
        else
            eri_kernel<125><<<blocks, 128, 0, st>>>(n, nquart, pw, poff, pp, dord, dE, accurate);
        CCSD_LAUNCH_CHECK();
        if (!device_out)
            CCSD_CUDA(cudaMemcpyAsync(eri, dE, sizeof(double) * nn * nn, cudaMemcpyDeviceToHost, st));
    }
    if (!device_out) {
        if (S) CCSD_CUDA(cudaMemcpyAsync(S, d_S.p, sizeof(double) * nn, cudaMemcpyDeviceToHost, st));
        if (T) CCSD_CUDA(cudaMemcpyAsync(T, d_L.p, sizeof(double) * nn, cudaMemcpyDeviceToHost, st));
        if (V) CCSD_CUDA(cudaMemcpyAsync(V, d_N.p, sizeof(double) * nn, cudaMemcpyDeviceToHost, st));
    }
    CCSD_CUDA(cudaStreamSynchronize(st));
}

}  // namespace ccsd

extern "C" int ccsd_ao_integrals(const ccsd_basis *basis, double *S, double *T, double *V, double *eri,
                                 double *e_nuc, int32_t device_outputs, void *stream) {
    try {
        ccsd::set_last_error("");
        if (!basis) throw ccsd::Error(CCSD_ERR_INVALID_ARG, "ccsd_ao_integrals: basis is NULL");
        int ndev = 0;
        if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
            cudaGetLastError();
            throw ccsd::Error(CCSD_ERR_NO_DEVICE, "no CUDA device: this engine has no CPU path");
        }
        ccsd::ao_integrals(*basis, S, T, V, eri, e_nuc, device_outputs != 0, (cudaStream_t)stream);
        return CCSD_OK;
    } catch (const ccsd::Error &e) {
        ccsd::set_last_error(e.what());
        return e.code;
    } catch (const std::exception &e) {
        ccsd::set_last_error(e.what());
        return CCSD_ERR_CUDA;
    }
}
