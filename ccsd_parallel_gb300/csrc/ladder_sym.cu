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
#include <algorithm>
#include <cmath>

#include "common.h"
#include "fp64_ops.cuh"
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

// (p, q) with p >= q from a pair index P < 2^24 (tile and occupied pairs)
__device__ __forceinline__ void untri32(int P, int &p, int &q) {
    int x = (int)((sqrtf(8.0f * (float)P + 1.0f) - 1.0f) * 0.5f);
    while (x * (x + 1) / 2 > P) --x;
    while ((x + 1) * (x + 2) / 2 <= P) ++x;
    p = x;
    q = P - x * (x + 1) / 2;
}

// The same packs by tiles: a block takes one pair i >= j and one 32 x 32 tile (C, D), C >= D,
// of (c, d).  tau[i][j] and tau[j][i] are read at tile (C, D) along d directly and at tile
// (D, C) along c into shared memory, so every element is read once and the pair rows are
// written along d.  Pair and tile indices are decoded per tile.
// I: int32_t when every offset of tau and the pair arrays is below 2^31 (64-bit integer
// arithmetic issues on the FP64 pipe on this part), else int64_t
template <typename I>
__global__ void __launch_bounds__(256) tau_sym_tiled_kernel(int o, int v, const double *__restrict__ tau,
                                                            double *__restrict__ tp, double *__restrict__ tm) {
    __shared__ double s2[32][33], s3[32][33];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int nt = (v + 31) / 32, ntt = nt * (nt + 1) / 2, To = o * (o + 1) / 2;
    const I Tv = (I)v * (v + 1) / 2, Tmv = (I)v * (v - 1) / 2;
    const I v2 = (I)v * v;
    const int nblk = To * ntt;
    for (int t = blockIdx.x; t < nblk; t += gridDim.x) {
        const int I_ = t / ntt;
        int i, j, C, D;
        untri32(I_, i, j);
        untri32(t % ntt, C, D);
        const double *tij = tau + ((I)i * o + j) * v2;
        const double *tji = tau + ((I)j * o + i) * v2;
        for (int q = ty; q < 32; q += 8) {  // s2[d][c] = tau[i][j][d][c], s3[d][c] = tau[j][i][d][c]
            const int d = D * 32 + q, c = C * 32 + tx;
            const bool in = d < v && c < v;
            s2[q][tx] = in ? tij[(I)d * v + c] : 0.0;
            s3[q][tx] = in ? tji[(I)d * v + c] : 0.0;
        }
        __syncthreads();
        const int d = D * 32 + tx;
        const I rowp = (I)I_ * Tv;
        const I rowm = i > j ? ((I)i * (i - 1) / 2 + j) * Tmv : 0;
        for (int q = ty; q < 32; q += 8) {
            const int c = C * 32 + q;
            if (c < v && d < v && d <= c) {
                const double x1 = tij[(I)c * v + d], x2 = s2[tx][q];
                const double x3 = s3[tx][q], x4 = tji[(I)c * v + d];
                // four FP64 additions; the quarter is taken on the exponent field
                const double u = x1 + x3, w = x2 + x4;
                tp[rowp + (I)c * (c + 1) / 2 + d] = mul_pow2(u + w, -2);
                if (i > j && c > d) tm[rowm + (I)c * (c - 1) / 2 + d] = mul_pow2(u - w, -2);
            }
        }
        __syncthreads();
    }
}

// The unpack by tiles of (a, b) for each (i, j): where a >= b the pair rows are read along
// b directly; where a < b (tiles A <= B) they are read along a into shared memory.
template <typename I>
__global__ void __launch_bounds__(256) ladder_unpack_tiled_kernel(int o, int v, const double *__restrict__ sp,
                                                                  const double *__restrict__ sm,
                                                                  double *__restrict__ R) {
    __shared__ double s_p[32][33], s_m[32][33];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int nt = (v + 31) / 32, ntiles = o * o * nt * nt;
    const I Tv = (I)v * (v + 1) / 2, Tmv = (I)v * (v - 1) / 2;
    const I v2 = (I)v * v;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        int r = t;
        const int B = r % nt;
        r /= nt;
        const int A = r % nt;
        r /= nt;
        const int j = r % o, i = r / o;
        const int i1 = max(i, j), j1 = min(i, j);
        const int sij = i > j ? 1 : (i < j ? -1 : 0);
        const I rowp = ((I)i1 * (i1 + 1) / 2 + j1) * Tv;
        const I rowm = sij ? ((I)i1 * (i1 - 1) / 2 + j1) * Tmv : 0;
        if (A <= B) {  // elements a < b: S at pair (b, a), read along a
            for (int q = ty; q < 32; q += 8) {
                const int b = B * 32 + q, a = A * 32 + tx;
                const bool in = b < v && a < v && b >= a;
                s_p[q][tx] = in ? sp[rowp + (I)b * (b + 1) / 2 + a] : 0.0;
                s_m[q][tx] = (in && sij && b > a) ? sm[rowm + (I)b * (b - 1) / 2 + a] : 0.0;
            }
        }
        __syncthreads();
        const int b = B * 32 + tx;
        double *Rij = R + ((I)i * o + j) * v2;
        for (int q = ty; q < 32; q += 8) {
            const int a = A * 32 + q;
            if (a >= v || b >= v) continue;
            double s;
            if (a >= b) {
                s = sp[rowp + (I)a * (a + 1) / 2 + b];
                if (sij && a > b) s += sij * sm[rowm + (I)a * (a - 1) / 2 + b];
            } else {
                s = s_p[tx][q];
                if (sij) s += -sij * s_m[tx][q];
            }
            Rij[(I)a * v + b] += s;
        }
        __syncthreads();
    }
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

// The same pair form for the other contractions over a (c,d) or (k,l) pair of tau, with the
// ladder's tau+- (the halves of tau symmetrised over its partners, above):
// - Z[i][j][k][a] = sum_cd (kd|ac) tau[ij,cd] (o^3 v^3) and X[k][l][i][j] = sum_cd (kc|ld)
//   tau[ij,cd] (o^4 v^2).  With V[r][c,d] the integral row r = (k,a) or (k,l):
//     Ps[tri(i,j)][r]  = sum_{c>=d} V+[r][tri(c,d)]  tau+[tri(i,j)][tri(c,d)]
//     Pa[stri(i,j)][r] = sum_{c>d}  V-[r][stri(c,d)] tau-[stri(i,j)][stri(c,d)]
//     P[i][j] = Ps + Pa,  P[j][i] = Ps - Pa  (i > j),  P[i][i] = Ps
//   with V+ = V[c,d] + V[d,c] (c > d), V[c,c] (c = d), V- = V[c,d] - V[d,c]: the plain
//   form on the symmetrised tau, half of its operations.
// - the hh ladder S[ij,ab] = sum_kl W[kl,ij] tau[kl,ab] adds to the pp ladder's halves:
//     S+[tri(i,j)][tri(a,b)]   += sum_{k>=l} W+[tri(i,j)][tri(k,l)]   tau+[tri(k,l)][tri(a,b)]
//     S-[stri(i,j)][stri(a,b)] += sum_{k>l}  W-[stri(i,j)][stri(k,l)] tau-[stri(k,l)][stri(a,b)]
//   with W+- the (k,l) packs of W[.,ij] as above (tau+- of symmetric amplitudes are also
//   the (k,l)-symmetric and -antisymmetric halves of tau[kl,ab]), a quarter of 2 o^4 v^2.
//
// Row packs of V[r][c,d] for r < rows: V+[r][tri(c,d)] = V[c,d] + V[d,c] (c > d), V[c,c]
// (c = d); V-[r][stri(c,d)] = V[c,d] - V[d,c].  Row r = (r1, r2), r2 < n2, starts at
// r1 s1 + r2 s2 of a matrix Y[p][q] = base[p sp + q]; V[c,d] = Y[d][c] when yt is set
// (ovvv[k][d][a][c] = (kd|ac) for Z), else Y[c][d] (ovov[k][c][l][d] = (kc|ld) for X).
// Built once.  A block takes one row and one 32 x 32 tile (C, D), C >= D, reads tile
// (D, C) along q into shared memory (the transposed reads Y[d][c]) and tile (C, D) along
// d directly (Y[c][d]), and writes rows of consecutive d.  Every Y element is read once.
__global__ void __launch_bounds__(256) row_pair_pack_kernel(int64_t rows, int n2, int64_t s1, int64_t s2, int64_t sp,
                                                            int v, int yt, const double *__restrict__ base,
                                                            double *__restrict__ vp, double *__restrict__ vm) {
    __shared__ double s[32][33];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int nt = (v + 31) / 32;
    const int64_t ntt = (int64_t)nt * (nt + 1) / 2;
    const int64_t Tv = (int64_t)v * (v + 1) / 2, Tmv = (int64_t)v * (v - 1) / 2;
    for (int64_t t = blockIdx.x; t < rows * ntt; t += gridDim.x) {
        const int64_t r = t / ntt;
        int C, D;
        untri(t % ntt, C, D);
        const double *Y = base + (r / n2) * s1 + (r % n2) * s2;
        for (int q = ty; q < 32; q += 8) {  // s[q][tx] = Y[d = D*32 + q][c = C*32 + tx]
            const int d = D * 32 + q, c = C * 32 + tx;
            s[q][tx] = (d < v && c < v) ? Y[(int64_t)d * sp + c] : 0.0;
        }
        __syncthreads();
        const int d = D * 32 + tx;
        for (int q = ty; q < 32; q += 8) {
            const int c = C * 32 + q;
            if (c < v && d <= c) {
                const double ydc = s[tx][q], ycd = Y[(int64_t)c * sp + d];
                const double x = yt ? ydc : ycd, y = yt ? ycd : ydc;  // V[c,d], V[d,c]
                vp[r * Tv + (int64_t)c * (c + 1) / 2 + d] = c > d ? x + y : x;
                if (c > d) vm[r * Tmv + (int64_t)c * (c - 1) / 2 + d] = x - y;
            }
        }
        __syncthreads();
    }
}

// X[r][i][j] = Xs[r][tri(i,j)] + sgn(i - j) Xa[r][stri(i,j)] for r < o^2 (the pair index
// inner: the pair-form X of the o^4 product); xa may be null (no strict pairs)
__global__ void __launch_bounds__(256) x_pair_unpack_kernel(int o, const double *__restrict__ xs,
                                                            const double *__restrict__ xa, double *__restrict__ X) {
    const int64_t To = (int64_t)o * (o + 1) / 2, Tmo = (int64_t)o * (o - 1) / 2, n = (int64_t)o * o * o * o;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        const int j = (int)(e % o), i = (int)((e / o) % o);
        const int64_t r = e / ((int64_t)o * o);
        const int i1 = max(i, j), j1 = min(i, j);
        double x = xs[r * To + (int64_t)i1 * (i1 + 1) / 2 + j1];
        if (xa && i != j) {
            const double a = xa[r * Tmo + (int64_t)i1 * (i1 - 1) / 2 + j1];
            x = i > j ? x + a : x - a;
        }
        X[e] = x;
    }
}

// Pair packs of the hh-ladder intermediate W[k][l][i][j] over (k, l) for the rows i >= j:
// wp[tri(i,j)][tri(k,l)] = W[kl,ij] + W[lk,ij] (k > l), W[kk,ij]; wm[stri(i,j)][stri(k,l)] =
// W[kl,ij] - W[lk,ij] (i > j, k > l).  One thread per wp element.
__global__ void __launch_bounds__(256) oooo_pair_pack_kernel(int o, const double *__restrict__ W,
                                                             double *__restrict__ wp, double *__restrict__ wm) {
    const int64_t To = (int64_t)o * (o + 1) / 2, Tmo = (int64_t)o * (o - 1) / 2, o2 = (int64_t)o * o;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < To * To; e += (int64_t)gridDim.x * blockDim.x) {
        int i, j, k, l;
        untri(e / To, i, j);
        untri(e % To, k, l);
        const double x = W[((int64_t)k * o + l) * o2 + (int64_t)i * o + j];
        const double y = W[((int64_t)l * o + k) * o2 + (int64_t)i * o + j];
        wp[e] = k > l ? x + y : x;
        if (i > j && k > l) wm[stri(i, j) * Tmo + stri(k, l)] = x - y;
    }
}

// Z[i][j][n] = Zs[tri][n] + sgn(i - j) Za[stri][n] for n < o v (za may be null when there
// are no strict pairs on one side).  Blocks along y take rows (i, j), whose offsets are formed
// once per row; the offsets within a row (n < 2^31) are 32-bit.
__global__ void __launch_bounds__(256) z_pair_unpack_kernel(int o, int n, const double *__restrict__ zs,
                                                            const double *__restrict__ za, double *__restrict__ Z) {
    for (int row = blockIdx.y; row < o * o; row += gridDim.y) {
        const int i = row / o, j = row % o, i1 = max(i, j), j1 = min(i, j);
        const double *ps = zs + ((int64_t)i1 * (i1 + 1) / 2 + j1) * n;
        const double *pa = (za && i != j) ? za + ((int64_t)i1 * (i1 - 1) / 2 + j1) * n : nullptr;
        double *z = Z + (int64_t)row * n;
        for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x)
            z[c] = pa ? (i > j ? ps[c] + pa[c] : ps[c] - pa[c]) : ps[c];
    }
}

}  // namespace

// every offset of an o^2 v^2 array and of the tau+ pair array below 2^31
static bool small_offsets(int o, int v) {
    const int64_t n2 = (int64_t)o * o * v * v, np = (int64_t)o * (o + 1) / 2 * ((int64_t)v * (v + 1) / 2);
    return n2 < (1LL << 31) && np < (1LL << 31);
}

void k_tau_sym(int o, int v, const double *tau, double *tp, double *tm, cudaStream_t st) {
    const int64_t nt = (v + 31) / 32, blocks = (int64_t)o * (o + 1) / 2 * (nt * (nt + 1) / 2);
    if (blocks < (1LL << 30) && (int64_t)o * (o + 1) / 2 < (1 << 24)) {
        const int grid = (int)std::min<int64_t>(blocks, 152 * 8);
        if (small_offsets(o, v))
            tau_sym_tiled_kernel<int32_t><<<grid, 256, 0, st>>>(o, v, tau, tp, tm);
        else
            tau_sym_tiled_kernel<int64_t><<<grid, 256, 0, st>>>(o, v, tau, tp, tm);
    } else {
        const size_t n = (size_t)o * (o + 1) / 2 * ((size_t)v * (v + 1) / 2);
        tau_sym_kernel<<<blocks_for(n), 256, 0, st>>>(o, v, tau, tp, tm);
    }
    CCSD_LAUNCH_CHECK();
}

void k_tau_sym_adj(int o, int v, const double *tpb, const double *tmb, double *taub, cudaStream_t st) {
    tau_sym_adj_kernel<<<blocks_for((size_t)o * o * v * v), 256, 0, st>>>(o, v, tpb, tmb, taub);
    CCSD_LAUNCH_CHECK();
}

void k_ladder_unpack(int o, int v, const double *sp, const double *sm, double *R, cudaStream_t st) {
    const int64_t nt = (v + 31) / 32, tiles = (int64_t)o * o * nt * nt;
    if (tiles < (1LL << 30) && small_offsets(o, v))
        ladder_unpack_tiled_kernel<int32_t><<<(int)std::min<int64_t>(tiles, 152 * 8), 256, 0, st>>>(o, v, sp, sm, R);
    else if (tiles < (1LL << 30))
        ladder_unpack_tiled_kernel<int64_t><<<(int)std::min<int64_t>(tiles, 152 * 8), 256, 0, st>>>(o, v, sp, sm, R);
    else
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

static void row_pair_pack(int64_t rows, int n2, int64_t s1, int64_t s2, int64_t sp, int v, int yt,
                          const double *base, double *vp, double *vm, cudaStream_t st) {
    const int64_t nt = (v + 31) / 32, blocks = rows * (nt * (nt + 1) / 2);
    if (blocks == 0) return;
    row_pair_pack_kernel<<<(int)std::min<int64_t>(blocks, 152 * 8), 256, 0, st>>>(rows, n2, s1, s2, sp, v, yt, base,
                                                                                 vp, vm);
    CCSD_LAUNCH_CHECK();
}

void k_ovvv_pair_pack(int o, int v, const double *ovvv, double *vp, double *vm, cudaStream_t st) {
    // row (k, a) of Y[d][c] = ovvv[k][d][a][c]: k v^3 + a v, Y row stride v^2; V[c,d] = Y[d][c]
    const int64_t v2 = (int64_t)v * v;
    row_pair_pack((int64_t)o * v, v, v * v2, v, v2, v, 1, ovvv, vp, vm, st);
}

void k_ovov_pair_pack(int o, int v, const double *ovov, double *up, double *um, cudaStream_t st) {
    // row (k, l) of Y[c][d] = ovov[k][c][l][d]: k v o v + l v, Y row stride o v; U[c,d] = Y[c][d]
    const int64_t ov = (int64_t)o * v;
    row_pair_pack((int64_t)o * o, o, v * ov, v, ov, v, 0, ovov, up, um, st);
}

void k_x_pair_unpack(int o, const double *xs, const double *xa, double *X, cudaStream_t st) {
    const int64_t n = (int64_t)o * o * o * o;
    if (n == 0) return;
    x_pair_unpack_kernel<<<(int)std::min<int64_t>((n + 255) / 256, 152 * 8), 256, 0, st>>>(o, xs, xa, X);
    CCSD_LAUNCH_CHECK();
}

void k_oooo_pair_pack(int o, const double *W, double *wp, double *wm, cudaStream_t st) {
    const int64_t To = (int64_t)o * (o + 1) / 2;
    if (To == 0) return;
    oooo_pair_pack_kernel<<<(int)std::min<int64_t>((To * To + 255) / 256, 152 * 8), 256, 0, st>>>(o, W, wp, wm);
    CCSD_LAUNCH_CHECK();
}

void k_z_pair_unpack(int o, int v, const double *zs, const double *za, double *Z, cudaStream_t st) {
    const int n = o * v;
    if (n == 0) return;
    const dim3 grid((unsigned)std::min(4, (n + 255) / 256), (unsigned)std::min(o * o, 65535));
    z_pair_unpack_kernel<<<grid, 256, 0, st>>>(o, n, zs, za, Z);
    CCSD_LAUNCH_CHECK();
}

}  // namespace ccsd
