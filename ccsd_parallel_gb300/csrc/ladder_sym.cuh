// Pair-index helpers and per-element bodies of the pair-form ladder shared by
// the single-system kernels (ladder_sym.cu) and the grouped ones (grouped.cu).
// tri(p,q) = p(p+1)/2 + q for p >= q; stri(p,q) = p(p-1)/2 + q for p > q.
#pragma once

#include <cstdint>

namespace ccsd {
namespace pair {

__device__ __forceinline__ int64_t tri(int p, int q) { return (int64_t)p * (p + 1) / 2 + q; }
__device__ __forceinline__ int64_t stri(int p, int q) { return (int64_t)p * (p - 1) / 2 + q; }

// (p, q) with p >= q from a tri index
__device__ __forceinline__ void untri(int64_t P, int &p, int &q) {
    int x = (int)((sqrt(8.0 * (double)P + 1.0) - 1.0) * 0.5);
    while ((int64_t)x * (x + 1) / 2 > P) --x;
    while ((int64_t)(x + 1) * (x + 2) / 2 <= P) ++x;
    p = x;
    q = (int)(P - (int64_t)x * (x + 1) / 2);
}

__device__ __forceinline__ int sgn(int a, int b) { return a > b ? 1 : (a < b ? -1 : 0); }

// element idx < o(o+1)/2 * v(v+1)/2 of tau+ (and the matching tau- element)
__device__ __forceinline__ void tau_sym_elem(int o, int v, const double *__restrict__ tau, double *__restrict__ tp,
                                             double *__restrict__ tm, int64_t idx) {
    const int64_t Tv = (int64_t)v * (v + 1) / 2, Tmv = (int64_t)v * (v - 1) / 2;
    const int64_t v2 = (int64_t)v * v, ov2 = (int64_t)o * v2;
    const int64_t I = idx / Tv, Q = idx % Tv;
    int i, j, c, d;
    untri(I, i, j);
    untri(Q, c, d);
    const double x1 = tau[i * ov2 + j * v2 + (int64_t)c * v + d];
    const double x2 = tau[i * ov2 + j * v2 + (int64_t)d * v + c];
    const double x3 = tau[j * ov2 + i * v2 + (int64_t)d * v + c];
    const double x4 = tau[j * ov2 + i * v2 + (int64_t)c * v + d];
    const double u = x1 + x3, w = x2 + x4;  // the tiled kernel's order of additions
    tp[idx] = 0.25 * (u + w);
    if (i > j && c > d) tm[stri(i, j) * Tmv + stri(c, d)] = 0.25 * (u - w);
}

// element idx < o^2 v^2 of R[i][j][a][b] += S+ + sgn sgn S-
__device__ __forceinline__ void unpack_elem(int o, int v, const double *__restrict__ sp, const double *__restrict__ sm,
                                            double *__restrict__ R, int64_t idx) {
    const int64_t Tv = (int64_t)v * (v + 1) / 2, Tmv = (int64_t)v * (v - 1) / 2;
    const int b = (int)(idx % v);
    int64_t r = idx / v;
    const int a = (int)(r % v);
    r /= v;
    const int j = (int)(r % o);
    const int i = (int)(r / o);
    const int i1 = max(i, j), j1 = min(i, j), a1 = max(a, b), b1 = min(a, b);
    double s = sp[tri(i1, j1) * Tv + tri(a1, b1)];
    const int sg = sgn(i, j) * sgn(a, b);
    if (sg != 0) s += sg * sm[stri(i1, j1) * Tmv + stri(a1, b1)];
    R[idx] += s;
}

}  // namespace pair
}  // namespace ccsd
