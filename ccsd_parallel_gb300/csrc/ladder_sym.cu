// Symmetric / antisymmetric form of the particle-particle ladder.
//
//   S[ij,ab] = sum_cd W[ab,cd] tau[ij,cd],   W[a][b][c][d] = (ac|bd)
//
// With S[ij,ab] = S[ji,ba], tau[ij,cd] = tau[ji,dc] and W[ab,cd] = W[ba,dc],
// the halves S+- = (S[ij,ab] +- S[ij,ba]) / 2 need only i >= j, a >= b,
// c >= d:
//   S+[ij,ab] = sum_{c>=d} W+[ab,cd] tau+[ij,cd]   (i >= j, a >= b)
//   S-[ij,ab] = sum_{c>d}  W-[ab,cd] tau-[ij,cd]   (i >  j, a >  b)
// two contractions of about (v^2/2) x (o^2/2) x (v^2/2) each, a quarter of
// the 2 o^2 v^4 of the plain form.  Pair indices are lower-triangular:
// tri(p,q) = p(p+1)/2 + q (p >= q), stri(p,q) = p(p-1)/2 + q (p > q).
//
// The packs read all four symmetric partners of each element,
//   tau+ = (tau[ijcd] + tau[ijdc] + tau[jidc] + tau[jicd]) / 4, ...
//   W+   = f(c,d) + f(d,c) (c > d), f(c,c) (c = d), f(c,d) = (W[abcd] + W[badc]) / 2,
// so the map equals the plain ladder on symmetrised inputs: for symmetric
// inputs the result is the plain ladder's, and derivatives per input element
// equal the plain ladder's (whose derivative is itself symmetric).  Each
// pack/unpack has its transpose here for the adjoint sweep.
#include <cmath>

#include "common.h"
#include "ladder_sym.cuh"

namespace ccsd {

namespace {

using pair::sgn;
using pair::stri;
using pair::tri;
using pair::untri;

inline int blocks_for(size_t n) {
    size_t b = (n + 255) / 256;
    if (b > 8 * 152 * 4) b = 8 * 152 * 4;
    return b < 1 ? 1 : (int)b;
}

// tau+[tri(i,j)][tri(c,d)], tau-[stri(i,j)][stri(c,d)]; one thread per tau+ element
__global__ void tau_sym_kernel(int o, int v, const double *__restrict__ tau, double *__restrict__ tp,
                               double *__restrict__ tm) {
    const int64_t total = (int64_t)o * (o + 1) / 2 * ((int64_t)v * (v + 1) / 2);
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x)
        pair::tau_sym_elem(o, v, tau, tp, tm, idx);
}

// transpose of tau_sym: taubar[i,j,c,d] += cp tp_bar[..] + s/4 tm_bar[..]
__global__ void tau_sym_adj_kernel(int o, int v, const double *__restrict__ tpb, const double *__restrict__ tmb,
                                   double *__restrict__ taub) {
    const int64_t Tv = (int64_t)v * (v + 1) / 2, Tmv = (int64_t)v * (v - 1) / 2;
    const int64_t total = (int64_t)o * o * v * v;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int d = (int)(idx % v);
        int64_t r = idx / v;
        const int c = (int)(r % v);
        r /= v;
        const int j = (int)(r % o);
        const int i = (int)(r / o);
        const int i1 = max(i, j), j1 = min(i, j), c1 = max(c, d), d1 = min(c, d);
        const double cp = 0.25 * (i == j ? 2.0 : 1.0) * (c == d ? 2.0 : 1.0);
        double g = cp * tpb[tri(i1, j1) * Tv + tri(c1, d1)];
        const int s = sgn(i, j) * sgn(c, d);
        if (s != 0) g += 0.25 * s * tmb[stri(i1, j1) * Tmv + stri(c1, d1)];
        taub[idx] += g;
    }
}

// R[i,j,a,b] += S+[tri(i,j)-pair][tri(a,b)-pair] + sgn(i-j) sgn(a-b) S-[..][..]
// S+ is stored [I][P] (P fastest), S- [I'][P'].
__global__ void ladder_unpack_kernel(int o, int v, const double *__restrict__ sp, const double *__restrict__ sm,
                                     double *__restrict__ R) {
    const int64_t total = (int64_t)o * o * v * v;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x)
        pair::unpack_elem(o, v, sp, sm, R, idx);
}

// transpose of the unpack: S+bar[I][P] += sum of Rbar over the (up to) four
// index orders; S-bar[I'][P'] += signed sum.
__global__ void ladder_unpack_adj_kernel(int o, int v, const double *__restrict__ Rb, double *__restrict__ spb,
                                         double *__restrict__ smb) {
    const int64_t Tv = (int64_t)v * (v + 1) / 2, Tmv = (int64_t)v * (v - 1) / 2;
    const int64_t total = (int64_t)o * (o + 1) / 2 * Tv;
    const int64_t v2 = (int64_t)v * v, ov2 = (int64_t)o * v2;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t I = idx / Tv, P = idx % Tv;
        int i, j, a, b;
        untri(I, i, j);
        untri(P, a, b);
        const double r1 = Rb[i * ov2 + j * v2 + (int64_t)a * v + b];
        const double r2 = i != j ? Rb[j * ov2 + i * v2 + (int64_t)a * v + b] : 0.0;
        const double r3 = a != b ? Rb[i * ov2 + j * v2 + (int64_t)b * v + a] : 0.0;
        const double r4 = (i != j && a != b) ? Rb[j * ov2 + i * v2 + (int64_t)b * v + a] : 0.0;
        spb[idx] += (r1 + r2) + (r3 + r4);
        if (i > j && a > b) smb[stri(i, j) * Tmv + stri(a, b)] += (r1 - r2) - (r3 - r4);
    }
}

// W+[tri(a,b)][tri(c,d)] and W-[stri(a,b)][stri(c,d)] from W[a][b][c][d]
__global__ void w_sym_kernel(int v, const double *__restrict__ W, double *__restrict__ wp,
                             double *__restrict__ wm) {
    const int64_t Tv = (int64_t)v * (v + 1) / 2, Tmv = (int64_t)v * (v - 1) / 2;
    const int64_t total = Tv * Tv;
    const int64_t v2 = (int64_t)v * v;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t P = idx / Tv, Q = idx % Tv;
        int a, b, c, d;
        untri(P, a, b);
        untri(Q, c, d);
        const int64_t ab = ((int64_t)a * v + b) * v2, ba = ((int64_t)b * v + a) * v2;
        const double fcd = 0.5 * (W[ab + (int64_t)c * v + d] + W[ba + (int64_t)d * v + c]);
        if (c == d) {
            wp[idx] = fcd;
        } else {
            const double fdc = 0.5 * (W[ab + (int64_t)d * v + c] + W[ba + (int64_t)c * v + d]);
            wp[idx] = fcd + fdc;
            if (a > b) wm[stri(a, b) * Tmv + stri(c, d)] = fcd - fdc;
        }
    }
}

// The same by tiles: a block takes one pair a >= b and one 32 x 32 tile (C, D), C >= D, of
// (c, d); it reads W[a][b] and W[b][a] at tiles (C, D) and (D, C) along their rows into
// shared memory, so the transposed reads W[..][d][c] come from there, and writes W+/W-
// rows of consecutive d.  Each W element is read once.
constexpr int WT = 32;
__global__ void __launch_bounds__(256) w_sym_tiled_kernel(int v, const double *__restrict__ W,
                                                          double *__restrict__ wp, double *__restrict__ wm) {
    __shared__ double t_ab_cd[WT][WT + 1], t_ba_cd[WT][WT + 1], t_ab_dc[WT][WT + 1], t_ba_dc[WT][WT + 1];
    const int nt = (v + WT - 1) / WT;
    const int64_t ntt = (int64_t)nt * (nt + 1) / 2;
    const int64_t Tv = (int64_t)v * (v + 1) / 2, Tmv = (int64_t)v * (v - 1) / 2, v2 = (int64_t)v * v;
    const int64_t P = blockIdx.x / ntt;
    int a, b, C, D;
    untri(P, a, b);
    untri(blockIdx.x % ntt, C, D);
    const int64_t ab = ((int64_t)a * v + b) * v2, ba = ((int64_t)b * v + a) * v2;
    const int tx = threadIdx.x % WT, ty = threadIdx.x / WT;  // 32 x 8
    for (int r = ty; r < WT; r += 8) {
        const int c = C * WT + r, d = D * WT + tx;  // rows c of tile (C, D)
        const bool in = c < v && d < v;
        t_ab_cd[r][tx] = in ? W[ab + (int64_t)c * v + d] : 0.0;
        t_ba_cd[r][tx] = in ? W[ba + (int64_t)c * v + d] : 0.0;
        const int dr = D * WT + r, cc = C * WT + tx;  // rows d of tile (D, C)
        const bool in2 = dr < v && cc < v;
        t_ab_dc[r][tx] = in2 ? W[ab + (int64_t)dr * v + cc] : 0.0;
        t_ba_dc[r][tx] = in2 ? W[ba + (int64_t)dr * v + cc] : 0.0;
    }
    __syncthreads();
    for (int r = ty; r < WT; r += 8) {
        const int c = C * WT + r, d = D * WT + tx;
        if (c >= v || d >= v || d > c) continue;
        // W[ab][c][d], W[ba][d][c], W[ab][d][c], W[ba][c][d]
        const double fcd = 0.5 * (t_ab_cd[r][tx] + t_ba_dc[tx][r]);
        const int64_t out = P * Tv + tri(c, d);
        if (c == d) {
            wp[out] = fcd;
        } else {
            const double fdc = 0.5 * (t_ab_dc[tx][r] + t_ba_cd[r][tx]);
            wp[out] = fcd + fdc;
            if (a > b) wm[stri(a, b) * Tmv + stri(c, d)] = fcd - fdc;
        }
    }
}

// transpose of w_sym: Wbar[a,b,c,d] += cw W+bar[..] + s/2 W-bar[..]
__global__ void w_sym_adj_kernel(int v, const double *__restrict__ wpb, const double *__restrict__ wmb,
                                 double *__restrict__ Wb) {
    const int64_t Tv = (int64_t)v * (v + 1) / 2, Tmv = (int64_t)v * (v - 1) / 2;
    const int64_t total = (int64_t)v * v * v * v;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int d = (int)(idx % v);
        int64_t r = idx / v;
        const int c = (int)(r % v);
        r /= v;
        const int b = (int)(r % v);
        const int a = (int)(r / v);
        const int a1 = max(a, b), b1 = min(a, b), c1 = max(c, d), d1 = min(c, d);
        double g = (a == b ? 1.0 : 0.5) * wpb[tri(a1, b1) * Tv + tri(c1, d1)];
        const int s = sgn(a, b) * sgn(c, d);
        if (s != 0) g += 0.5 * s * wmb[stri(a1, b1) * Tmv + stri(c1, d1)];
        Wb[idx] += g;
    }
}

}  // namespace

void k_tau_sym(int o, int v, const double *tau, double *tp, double *tm, cudaStream_t st) {
    const size_t n = (size_t)o * (o + 1) / 2 * ((size_t)v * (v + 1) / 2);
    tau_sym_kernel<<<blocks_for(n), 256, 0, st>>>(o, v, tau, tp, tm);
    CCSD_LAUNCH_CHECK();
}

void k_tau_sym_adj(int o, int v, const double *tpb, const double *tmb, double *taub, cudaStream_t st) {
    tau_sym_adj_kernel<<<blocks_for((size_t)o * o * v * v), 256, 0, st>>>(o, v, tpb, tmb, taub);
    CCSD_LAUNCH_CHECK();
}

void k_ladder_unpack(int o, int v, const double *sp, const double *sm, double *R, cudaStream_t st) {
    ladder_unpack_kernel<<<blocks_for((size_t)o * o * v * v), 256, 0, st>>>(o, v, sp, sm, R);
    CCSD_LAUNCH_CHECK();
}

void k_ladder_unpack_adj(int o, int v, const double *Rb, double *spb, double *smb, cudaStream_t st) {
    const size_t n = (size_t)o * (o + 1) / 2 * ((size_t)v * (v + 1) / 2);
    ladder_unpack_adj_kernel<<<blocks_for(n), 256, 0, st>>>(o, v, Rb, spb, smb);
    CCSD_LAUNCH_CHECK();
}

void k_w_sym(int v, const double *W, double *wp, double *wm, cudaStream_t st) {
    const int64_t nt = (v + WT - 1) / WT, blocks = (int64_t)v * (v + 1) / 2 * (nt * (nt + 1) / 2);
    if (blocks <= 0x7fffffffLL) {
        w_sym_tiled_kernel<<<(unsigned)blocks, 256, 0, st>>>(v, W, wp, wm);
    } else {
        const size_t n = ((size_t)v * (v + 1) / 2) * ((size_t)v * (v + 1) / 2);
        w_sym_kernel<<<blocks_for(n), 256, 0, st>>>(v, W, wp, wm);
    }
    CCSD_LAUNCH_CHECK();
}

void k_w_sym_adj(int v, const double *wpb, const double *wmb, double *Wb, cudaStream_t st) {
    w_sym_adj_kernel<<<blocks_for((size_t)v * v * v * v), 256, 0, st>>>(v, wpb, wmb, Wb);
    CCSD_LAUNCH_CHECK();
}

}  // namespace ccsd
