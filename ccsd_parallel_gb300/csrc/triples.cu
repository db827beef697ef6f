// CCSDT-1a triples (the reference's CCSDT method Method_Nr 1, ccsdt.cpp:735-1318)
// on top of the closed-shell CCSD engine, in the reference's spin-orbital form:
// spin orbital P = 2p + spin (alpha/beta interleaved, ccsdt.cpp:1466-1478).
//
//   t3[a][b][c][i][j][k] = [P(a/bc) P(k/ij) Y - P(c/ab) P(i/jk) Z] / D3
//   Y[abc][ijk] = sum_e t2(a,e)(i,j) <bc||ek>,  Z[abc][ijk] = sum_m t2(a,b)(i,m) <mc||jk>
//
// Y and Z are contractions (engine kernels); this file builds the
// spin-orbital integral blocks from the spatial ones, expands the spatial T2
// into spin orbitals, and assembles T3 (both antisymmetrisers and D3 in one
// pass, one thread per element, spin-forbidden elements left at zero).
// Sizes: O = 2 nocc, V = 2 nvir.
#include "common.h"

namespace ccsd {

namespace {

inline int blocks_for(size_t n) {
    size_t b = (n + 255) / 256;
    if (b > 8 * 152 * 4) b = 8 * 152 * 4;
    return b < 1 ? 1 : (int)b;
}

// spatial chemist blocks: ovov[i][a][j][b], ovoo[i][a][j][k], ovvv[i][a][b][c], and for the
// CCSDT-3 blocks oovv[i][j][a][b], oooo[i][j][k][l], wv[a][b][c][d] = (ac|bd)
struct Blocks {
    int o, v;
    const double *ovov, *ovoo, *ovvv, *oovv, *oooo, *wv;
    __device__ double OOVV(int i, int j, int a, int b) const {
        return oovv[(((int64_t)i * o + j) * v + a) * v + b];
    }
    __device__ double OOOO(int i, int j, int k, int l) const {
        return oooo[(((int64_t)i * o + j) * o + k) * o + l];
    }
    __device__ double WV(int a, int b, int c, int d) const {  // (ac|bd)
        return wv[(((int64_t)a * v + b) * v + c) * v + d];
    }
    __device__ double OVOV(int i, int a, int j, int b) const {
        return ovov[(((int64_t)i * v + a) * o + j) * v + b];
    }
    __device__ double OVOO(int i, int a, int j, int k) const {
        return ovoo[(((int64_t)i * v + a) * o + j) * o + k];
    }
    __device__ double OVVV(int i, int a, int b, int c) const {
        return ovvv[(((int64_t)i * v + a) * v + b) * v + c];
    }
};

// <PQ||RS> = (pr|qs) d(sp,sr) d(sq,ss) - (ps|qr) d(sp,ss) d(sq,sr), per block kind:
//   0: vvvo [b][c][e][k] = (be|ck) - (bk|ce)
//   1: ovoo [m][c][j][k] = (mj|ck) - (mk|cj)
//   2: oovv [j][k][b][c] = (jb|kc) - (jc|kb)
//   3: vovv [b][k][c][d] = (bc|kd) - (bd|kc)
//   4: ooov [k][m][j][c] = (kj|mc) - (kc|mj)
//   5: voov [a][l][i][d] = (ai|ld) - (ad|li)
//   6: oooo [m][l][i][j] = (mi|lj) - (mj|li)
//   7: vvvv [a][b][e][d] = (ae|bd) - (ad|be)
__global__ void so_block_kernel(int kind, Blocks B, double *out) {
    const int O = 2 * B.o, V = 2 * B.v;
    int e0, e1, e2, e3;  // extents of the four indices
    switch (kind) {
        case 0: e0 = V; e1 = V; e2 = V; e3 = O; break;
        case 1: e0 = O; e1 = V; e2 = O; e3 = O; break;
        case 2: e0 = O; e1 = O; e2 = V; e3 = V; break;
        case 3: e0 = V; e1 = O; e2 = V; e3 = V; break;
        case 4: e0 = O; e1 = O; e2 = O; e3 = V; break;
        case 5: e0 = V; e1 = O; e2 = O; e3 = V; break;
        case 6: e0 = O; e1 = O; e2 = O; e3 = O; break;
        default: e0 = V; e1 = V; e2 = V; e3 = V; break;
    }
    const int64_t total = (int64_t)e0 * e1 * e2 * e3;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int P3 = (int)(idx % e3);
        int64_t r = idx / e3;
        const int P2 = (int)(r % e2);
        r /= e2;
        const int P1 = (int)(r % e1);
        const int P0 = (int)(r / e1);
        const int p0 = P0 >> 1, p1 = P1 >> 1, p2 = P2 >> 1, p3 = P3 >> 1;
        const int s0 = P0 & 1, s1 = P1 & 1, s2 = P2 & 1, s3 = P3 & 1;
        double d = 0.0, x = 0.0;
        switch (kind) {
            case 0:  // <bc||ek>: (be|ck) = ovvv[k][c][b][e], (bk|ce) = ovvv[k][b][c][e]
                if (s0 == s2 && s1 == s3) d = B.OVVV(p3, p1, p0, p2);
                if (s0 == s3 && s1 == s2) x = B.OVVV(p3, p0, p1, p2);
                break;
            case 1:  // <mc||jk>: (mj|ck) = ovoo[k][c][m][j], (mk|cj) = ovoo[j][c][m][k]
                if (s0 == s2 && s1 == s3) d = B.OVOO(p3, p1, p0, p2);
                if (s0 == s3 && s1 == s2) x = B.OVOO(p2, p1, p0, p3);
                break;
            case 2:  // <jk||bc>: (jb|kc) = ovov[j][b][k][c], (jc|kb) = ovov[j][c][k][b]
                if (s0 == s2 && s1 == s3) d = B.OVOV(p0, p2, p1, p3);
                if (s0 == s3 && s1 == s2) x = B.OVOV(p0, p3, p1, p2);
                break;
            case 3:  // <bk||cd>: (bc|kd) = ovvv[k][d][b][c], (bd|kc) = ovvv[k][c][b][d]
                if (s0 == s2 && s1 == s3) d = B.OVVV(p1, p3, p0, p2);
                if (s0 == s3 && s1 == s2) x = B.OVVV(p1, p2, p0, p3);
                break;
            case 4:  // <km||jc>: (kj|mc) = ovoo[m][c][k][j], (kc|mj) = ovoo[k][c][m][j]
                if (s0 == s2 && s1 == s3) d = B.OVOO(p1, p3, p0, p2);
                if (s0 == s3 && s1 == s2) x = B.OVOO(p0, p3, p1, p2);
                break;
            case 5:  // <al||id>: (ai|ld) = ovov[i][a][l][d], (ad|li) = oovv[l][i][a][d]
                if (s0 == s2 && s1 == s3) d = B.OVOV(p2, p0, p1, p3);
                if (s0 == s3 && s1 == s2) x = B.OOVV(p1, p2, p0, p3);
                break;
            case 6:  // <ml||ij>: (mi|lj) = oooo[m][i][l][j], (mj|li) = oooo[m][j][l][i]
                if (s0 == s2 && s1 == s3) d = B.OOOO(p0, p2, p1, p3);
                if (s0 == s3 && s1 == s2) x = B.OOOO(p0, p3, p1, p2);
                break;
            default:  // <ab||ed>: (ae|bd) = wv[a][b][e][d], (ad|be) = wv[a][b][d][e]
                if (s0 == s2 && s1 == s3) d = B.WV(p0, p1, p2, p3);
                if (s0 == s3 && s1 == s2) x = B.WV(p0, p1, p3, p2);
                break;
        }
        out[idx] = d - x;
    }
}

// t2so[a][b][i][j] (spin orbitals) from the spatial t2[i][j][a][b]:
// t2[ij ab] d(sa,si) d(sb,sj) - t2[ji ab] d(sa,sj) d(sb,si)
__global__ void t2_spin_kernel(int o, int v, const double *__restrict__ t2, double *__restrict__ t2so) {
    const int O = 2 * o, V = 2 * v;
    const int64_t total = (int64_t)V * V * O * O;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int J = (int)(idx % O);
        int64_t r = idx / O;
        const int I = (int)(r % O);
        r /= O;
        const int Bv = (int)(r % V);
        const int A = (int)(r / V);
        const int a = A >> 1, b = Bv >> 1, i = I >> 1, j = J >> 1;
        const int sa = A & 1, sb = Bv & 1, si = I & 1, sj = J & 1;
        double val = 0.0;
        if (sa == si && sb == sj) val += t2[(((int64_t)i * o + j) * v + a) * v + b];
        if (sa == sj && sb == si) val -= t2[(((int64_t)j * o + i) * v + a) * v + b];
        t2so[idx] = val;
    }
}

// tauso[a][b][i][j] = t2so[a][b][i][j] + t1so[a][i] t1so[b][j] - t1so[a][j] t1so[b][i]
__global__ void tau_spin_kernel(int o, int v, const double *__restrict__ t2so, const double *__restrict__ t1so,
                                double *__restrict__ tauso) {
    const int O = 2 * o, V = 2 * v;
    const int64_t total = (int64_t)V * V * O * O;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int j = (int)(idx % O);
        int64_t r = idx / O;
        const int i = (int)(r % O);
        r /= O;
        const int b = (int)(r % V);
        const int a = (int)(r / V);
        tauso[idx] = t2so[idx] + (t1so[a * O + i] * t1so[b * O + j] - t1so[a * O + j] * t1so[b * O + i]);
    }
}

// t1so[a][i] (spin orbitals) from the spatial t1[i][a]: t1[i a] d(sa, si)
__global__ void t1_spin_kernel(int o, int v, const double *__restrict__ t1, double *__restrict__ t1so) {
    const int O = 2 * o, V = 2 * v;
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < V * O; idx += gridDim.x * blockDim.x) {
        const int I = idx % O, A = idx / O;
        t1so[idx] = ((A & 1) == (I & 1)) ? t1[(I >> 1) * v + (A >> 1)] : 0.0;
    }
}

// t3[a][b][c][i][j][k] = [P(a/bc) P(k/ij) Y - P(c/ab) P(i/jk) Z] / (D(a,i) + D(b,j) + D(c,k)),
// D(a,i) = f_ii - f_aa, with P(a/bc) = 1 - (ab) - (ac), P(k/ij) = 1 - (ik) - (jk),
// P(c/ab) = 1 - (ac) - (bc), P(i/jk) = 1 - (ij) - (ik) (ccsdt.cpp:1016-1058, 1235-1238)
__global__ void t3_assemble_kernel(int o, int v, const double *__restrict__ Y, const double *__restrict__ Z,
                                   const double *__restrict__ eo, const double *__restrict__ ev,
                                   double *__restrict__ t3) {
    const int O = 2 * o, V = 2 * v;
    const int64_t O3 = (int64_t)O * O * O;
    const int64_t total = (int64_t)V * V * V * O3;
    auto at = [&](const double *X, int a, int b, int c, int i, int j, int k) {
        return X[(((int64_t)a * V + b) * V + c) * O3 + ((int64_t)i * O + j) * O + k];
    };
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int k = (int)(idx % O);
        int64_t r = idx / O;
        const int j = (int)(r % O);
        r /= O;
        const int i = (int)(r % O);
        r /= O;
        const int c = (int)(r % V);
        r /= V;
        const int b = (int)(r % V);
        const int a = (int)(r / V);
        // spin conservation: Y, Z and t3 vanish unless abc and ijk carry the same
        // number of beta spins (20 of the 64 spin blocks); those stay at the zero
        // the buffer was set to
        if ((a & 1) + (b & 1) + (c & 1) != (i & 1) + (j & 1) + (k & 1)) continue;
        // P(a/bc) applied to each of P(k/ij)'s three index orders
        auto pa = [&](int p, int q, int s) {
            return at(Y, a, b, c, p, q, s) - at(Y, b, a, c, p, q, s) - at(Y, c, b, a, p, q, s);
        };
        const double y = pa(i, j, k) - pa(k, j, i) - pa(i, k, j);
        auto pc = [&](int p, int q, int s) {
            return at(Z, a, b, c, p, q, s) - at(Z, c, b, a, p, q, s) - at(Z, a, c, b, p, q, s);
        };
        const double z = pc(i, j, k) - pc(j, i, k) - pc(k, j, i);
        const double den = (eo[i >> 1] - ev[a >> 1]) + (eo[j >> 1] - ev[b >> 1]) + (eo[k >> 1] - ev[c >> 1]);
        t3[idx] = (y - z) / den;
    }
}

// The same T3 as t3_assemble_kernel, one CTA per virtual triple a < b < c
// (C(V,3) CTAs).  Y is antisymmetric in its last two virtual indices and Z in
// its first two, so P(a/bc) Y and P(c/ab) Z, and with them t3, are antisymmetric
// in abc: the CTA forms the O^3 slab of (a,b,c) and writes it, with the sign of
// each permutation, into the six slabs abc, acb, bac, bca, cab, cba.  Slabs with a
// repeated virtual index are zero and stay at the zero the buffer was set to.
//   ys[ijk] = Y[abc][ijk] - Y[bac][ijk] - Y[cba][ijk]     P(a/bc), slab-contiguous reads
//   zs[ijk] = Z[abc][ijk] - Z[cba][ijk] - Z[acb][ijk]     P(c/ab)
//   t3[abc][ijk] = ([ys(ijk) - ys(kji) - ys(ikj)] - [zs(ijk) - zs(jik) - zs(kji)]) / D3
// The occupied permutations read shared memory at stride s_i or s_j; both are odd
// (s_j = O + 1, s_i = O s_j + 1, O even), so a half-warp of doubles hits 16
// distinct bank pairs.  Every global read and write is of a contiguous slab.
__device__ __forceinline__ int64_t c3(int64_t n) { return n * (n - 1) * (n - 2) / 6; }

// -x by flipping the sign bit on the integer pipe (the same value as -x for every
// input), so the six signed copies of each element cost no FP64 issue slots.
__device__ __forceinline__ double negd(double x) {
    return __longlong_as_double(__double_as_longlong(x) ^ (long long)0x8000000000000000ULL);
}

// Single-precision estimates (FP32 issue is cheap, FP64 is not); the integer loops
// make the result exact.
__device__ __forceinline__ void decode_triple(int64_t t, int &a, int &b, int &c) {
    c = (int)cbrtf(6.0f * (float)t);
    if (c < 2) c = 2;
    while (c3(c + 1) <= t) ++c;
    while (c > 2 && c3(c) > t) --c;
    const int64_t r = t - c3(c);
    b = (int)sqrtf(2.0f * (float)r);
    if (b < 1) b = 1;
    while ((int64_t)(b + 1) * b / 2 <= r) ++b;
    while (b > 1 && (int64_t)b * (b - 1) / 2 > r) --b;
    a = (int)(r - (int64_t)b * (b - 1) / 2);
}

__global__ void __launch_bounds__(256) t3_assemble_slab_kernel(int o, int v, const double *__restrict__ Y,
                                                               const double *__restrict__ Z,
                                                               const double *__restrict__ eo,
                                                               const double *__restrict__ ev,
                                                               double *__restrict__ t3) {
    extern __shared__ double sm[];
    const int O = 2 * o, V = 2 * v;
    const int O3 = O * O * O, sj = O + 1, si = O * sj + 1;
    double *ys = sm, *zs = sm + (size_t)O * si;
    // blockIdx.x -> (a < b < c): c3(c) <= t < c3(c + 1), then r = t - c3(c) = b(b-1)/2 + a
    int a, b, c;
    decode_triple(blockIdx.x, a, b, c);
    auto slab = [&](int x, int y, int z) { return (((int64_t)x * V + y) * V + z) * O3; };
    const double *y0 = Y + slab(a, b, c), *y1 = Y + slab(b, a, c), *y2 = Y + slab(c, b, a);
    const double *z0 = Z + slab(a, b, c), *z1 = Z + slab(c, b, a), *z2 = Z + slab(a, c, b);
    for (int e = threadIdx.x; e < O3; e += blockDim.x) {
        const int k = e % O, j = (e / O) % O, i = e / (O * O);
        const int p = i * si + j * sj + k;
        ys[p] = (y0[e] - y1[e]) - y2[e];
        zs[p] = (z0[e] - z1[e]) - z2[e];
    }
    __syncthreads();
    const int64_t s_abc = slab(a, b, c), s_acb = slab(a, c, b), s_bac = slab(b, a, c);
    const int64_t s_bca = slab(b, c, a), s_cab = slab(c, a, b), s_cba = slab(c, b, a);
    const double fa = ev[a >> 1], fb = ev[b >> 1], fc = ev[c >> 1];
    for (int e = threadIdx.x; e < O3; e += blockDim.x) {
        const int k = e % O, j = (e / O) % O, i = e / (O * O);
        const double y = (ys[i * si + j * sj + k] - ys[k * si + j * sj + i]) - ys[i * si + k * sj + j];
        const double z = (zs[i * si + j * sj + k] - zs[j * si + i * sj + k]) - zs[k * si + j * sj + i];
        const double den = ((eo[i >> 1] - fa) + (eo[j >> 1] - fb)) + (eo[k >> 1] - fc);
        const double u = (y - z) / den;
        const double nu_ = negd(u);
        t3[s_abc + e] = u;
        t3[s_acb + e] = nu_;
        t3[s_bac + e] = nu_;
        t3[s_bca + e] = u;
        t3[s_cab + e] = u;
        t3[s_cba + e] = nu_;
    }
}

// The kernel above spends about 30 FP64 instructions on every element, and FP64
// issue is GB300's narrow resource (about 0.6 T instructions/s for the whole
// GPU).  This form does the same work with far fewer: t3 is also antisymmetric
// in ijk (Y in ij, Z in jk), so only i < j < k are evaluated and the six orders
// filled with signs in a shared-memory output slab; elements whose occupied spins
// do not balance the virtual ones (both sides must carry the same number of beta
// spins) are zero and skip their loads and arithmetic.  Phases:
//   1. ys, zs as above (spin-allowed elements only), output slab us = 0
//   2. i < j < k: u = ([ys(ijk) - ys(kji) - ys(ikj)] - [zs(ijk) - zs(jik) - zs(kji)]) / D3,
//      us at the six orders of ijk with their signs
//   3. us written to the six slabs of abc with their signs (contiguous)
template <bool M3>
__global__ void __launch_bounds__(256) t3_assemble_unique_kernel(int o, int v, const double *__restrict__ Y,
                                                                 const double *__restrict__ Z,
                                                                 const double *__restrict__ Q12,
                                                                 const double *__restrict__ Q13,
                                                                 const double *__restrict__ eo,
                                                                 const double *__restrict__ ev,
                                                                 double *__restrict__ t3) {
    // M3 (CCSDT-2): ws also carries P(abc) Q12 (both under P(i/jk)), and qs = P(a/bc) Q13
    // under the full P(ijk).  Without M3, ws = -P(c/ab) Z and the arithmetic is that of
    // [P(k/ij) ys - P(i/jk) zs] exactly.
    extern __shared__ double sm[];
    const int O = 2 * o, V = 2 * v;
    const int O3 = O * O * O, sj = O + 1, si = O * sj + 1, P = O * si;
    double *ys = sm, *ws = sm + P, *us = sm + 2 * P, *qs = sm + 3 * P;
    int a, b, c;
    decode_triple(blockIdx.x, a, b, c);
    const int sv = (a & 1) + (b & 1) + (c & 1);
    auto slab = [&](int x, int y, int z) { return (((int64_t)x * V + y) * V + z) * O3; };
    const double *y0 = Y + slab(a, b, c), *y1 = Y + slab(b, a, c), *y2 = Y + slab(c, b, a);
    const double *z0 = Z + slab(a, b, c), *z1 = Z + slab(c, b, a), *z2 = Z + slab(a, c, b);
    for (int e = threadIdx.x; e < O3; e += blockDim.x) {
        const int k = e % O, j = (e / O) % O, i = e / (O * O);
        const int p = i * si + j * sj + k;
        double yv = 0.0, wv = 0.0, qv = 0.0;
        if ((i & 1) + (j & 1) + (k & 1) == sv) {
            yv = (y0[e] - y1[e]) - y2[e];
            wv = negd((z0[e] - z1[e]) - z2[e]);
            if (M3) {
                const double q = ((((Q12[slab(a, b, c) + e] - Q12[slab(b, a, c) + e]) - Q12[slab(c, b, a) + e]) -
                                   Q12[slab(a, c, b) + e]) + Q12[slab(b, c, a) + e]) + Q12[slab(c, a, b) + e];
                wv = q + wv;
                qv = (Q13[slab(a, b, c) + e] - Q13[slab(b, a, c) + e]) - Q13[slab(c, b, a) + e];
            }
        }
        ys[p] = yv;
        ws[p] = wv;
        us[p] = 0.0;
        if (M3) qs[p] = qv;
    }
    __syncthreads();
    const double fa = ev[a >> 1], fb = ev[b >> 1], fc = ev[c >> 1];
    const int nu = O * (O - 1) * (O - 2) / 6;
    for (int t = threadIdx.x; t < nu; t += blockDim.x) {
        int i, j, k;
        decode_triple(t, i, j, k);
        double u = 0.0;
        if ((i & 1) + (j & 1) + (k & 1) == sv) {
            const double y = (ys[i * si + j * sj + k] - ys[k * si + j * sj + i]) - ys[i * si + k * sj + j];
            const double w = (ws[i * si + j * sj + k] - ws[j * si + i * sj + k]) - ws[k * si + j * sj + i];
            double num = y + w;
            if (M3) {
                const double q = ((((qs[i * si + j * sj + k] - qs[j * si + i * sj + k]) - qs[k * si + j * sj + i]) -
                                   qs[i * si + k * sj + j]) + qs[j * si + k * sj + i]) + qs[k * si + i * sj + j];
                num = num + q;
            }
            const double den = ((eo[i >> 1] - fa) + (eo[j >> 1] - fb)) + (eo[k >> 1] - fc);
            u = num / den;
        }
        const double nu_ = negd(u);
        us[i * si + j * sj + k] = u;
        us[i * si + k * sj + j] = nu_;
        us[j * si + i * sj + k] = nu_;
        us[j * si + k * sj + i] = u;
        us[k * si + i * sj + j] = u;
        us[k * si + j * sj + i] = nu_;
    }
    __syncthreads();
    const int64_t s_abc = slab(a, b, c), s_acb = slab(a, c, b), s_bac = slab(b, a, c);
    const int64_t s_bca = slab(b, c, a), s_cab = slab(c, a, b), s_cba = slab(c, b, a);
    for (int e = threadIdx.x; e < O3; e += blockDim.x) {
        const int k = e % O, j = (e / O) % O, i = e / (O * O);
        const double u = us[i * si + j * sj + k];
        const double nu_ = negd(u);
        t3[s_abc + e] = u;
        t3[s_acb + e] = nu_;
        t3[s_bac + e] = nu_;
        t3[s_bca + e] = u;
        t3[s_cab + e] = u;
        t3[s_cba + e] = nu_;
    }
}

// The CCSDT-2 numerator element by element (any O): global reads of every permuted
// operand, for O^3 slabs beyond shared memory or V < 3.
__global__ void t3_assemble_m3_kernel(int o, int v, const double *__restrict__ Y, const double *__restrict__ Z,
                                      const double *__restrict__ Q12, const double *__restrict__ Q13,
                                      const double *__restrict__ eo, const double *__restrict__ ev,
                                      double *__restrict__ t3) {
    const int O = 2 * o, V = 2 * v;
    const int64_t O3 = (int64_t)O * O * O;
    const int64_t total = (int64_t)V * V * V * O3;
    auto at = [&](const double *X, int a, int b, int c, int i, int j, int k) {
        return X[(((int64_t)a * V + b) * V + c) * O3 + ((int64_t)i * O + j) * O + k];
    };
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int k = (int)(idx % O);
        int64_t r = idx / O;
        const int j = (int)(r % O);
        r /= O;
        const int i = (int)(r % O);
        r /= O;
        const int c = (int)(r % V);
        r /= V;
        const int b = (int)(r % V);
        const int a = (int)(r / V);
        if ((a & 1) + (b & 1) + (c & 1) != (i & 1) + (j & 1) + (k & 1)) continue;
        auto pa = [&](int p, int q, int s) {
            return (at(Y, a, b, c, p, q, s) - at(Y, b, a, c, p, q, s)) - at(Y, c, b, a, p, q, s);
        };
        const double y = (pa(i, j, k) - pa(k, j, i)) - pa(i, k, j);
        auto pw = [&](int p, int q, int s) {
            const double z = (at(Z, a, b, c, p, q, s) - at(Z, c, b, a, p, q, s)) - at(Z, a, c, b, p, q, s);
            const double q12 = ((((at(Q12, a, b, c, p, q, s) - at(Q12, b, a, c, p, q, s)) - at(Q12, c, b, a, p, q, s)) -
                                 at(Q12, a, c, b, p, q, s)) + at(Q12, b, c, a, p, q, s)) + at(Q12, c, a, b, p, q, s);
            return q12 + negd(z);
        };
        const double w = (pw(i, j, k) - pw(j, i, k)) - pw(k, j, i);
        auto pq = [&](int p, int q, int s) {
            return (at(Q13, a, b, c, p, q, s) - at(Q13, b, a, c, p, q, s)) - at(Q13, c, b, a, p, q, s);
        };
        const double qq = ((((pq(i, j, k) - pq(j, i, k)) - pq(k, j, i)) - pq(i, k, j)) + pq(j, k, i)) + pq(k, i, j);
        const double den = (eo[i >> 1] - ev[a >> 1]) + (eo[j >> 1] - ev[b >> 1]) + (eo[k >> 1] - ev[c >> 1]);
        t3[idx] = ((y + w) + qq) / den;
    }
}

size_t slab_smem_bytes(int o, int arrays) {
    const size_t O = 2 * (size_t)o, si = O * (O + 1) + 1;
    return arrays * O * si * sizeof(double);
}
constexpr size_t kSlabSmemMax = 227 * 1024;

template <typename Kern>
void opt_in_smem(Kern kern, int &configured) {  // the opt-in above 48 KB is per device function
    int dev = 0;
    CCSD_CUDA(cudaGetDevice(&dev));
    if (configured != dev) {
        CCSD_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSlabSmemMax));
        configured = dev;
    }
}

}  // namespace

void k_so_block(int kind, int o, int v, const double *ovov, const double *ovoo, const double *ovvv,
                const double *oovv, const double *oooo, const double *wv, double *out, cudaStream_t st) {
    Blocks B{o, v, ovov, ovoo, ovvv, oovv, oooo, wv};
    const size_t O = 2 * (size_t)o, V = 2 * (size_t)v;
    const size_t sizes[8] = {V * V * V * O, O * V * O * O, O * O * V * V, V * O * V * V,
                             O * O * O * V, V * O * O * V, O * O * O * O, V * V * V * V};
    so_block_kernel<<<blocks_for(sizes[kind]), 256, 0, st>>>(kind, B, out);
    CCSD_LAUNCH_CHECK();
}

void k_tau_spin(int o, int v, const double *t2so, const double *t1so, double *tauso, cudaStream_t st) {
    tau_spin_kernel<<<blocks_for((size_t)16 * o * o * v * v), 256, 0, st>>>(o, v, t2so, t1so, tauso);
    CCSD_LAUNCH_CHECK();
}

void k_t1_spin(int o, int v, const double *t1, double *t1so, cudaStream_t st) {
    t1_spin_kernel<<<blocks_for((size_t)4 * o * v), 256, 0, st>>>(o, v, t1, t1so);
    CCSD_LAUNCH_CHECK();
}

void k_t2_spin(int o, int v, const double *t2, double *t2so, cudaStream_t st) {
    t2_spin_kernel<<<blocks_for((size_t)16 * o * o * v * v), 256, 0, st>>>(o, v, t2, t2so);
    CCSD_LAUNCH_CHECK();
}

void k_t3_assemble(int o, int v, const double *Y, const double *Z, const double *Q12, const double *Q13,
                   const double *eo, const double *ev, double *t3, cudaStream_t st) {
    const int64_t V = 2 * (int64_t)v, triples = V * (V - 1) * (V - 2) / 6;
    static int configured_unique = -1, configured_unique3 = -1, configured_slab = -1;
    if (Q12) {  // CCSDT-2 terms
        if (V >= 3 && slab_smem_bytes(o, 4) <= kSlabSmemMax) {  // O <= 18
            opt_in_smem(t3_assemble_unique_kernel<true>, configured_unique3);
            t3_assemble_unique_kernel<true><<<(unsigned)triples, 256, slab_smem_bytes(o, 4), st>>>(o, v, Y, Z, Q12, Q13,
                                                                                                 eo, ev, t3);
        } else {
            const size_t n = (size_t)64 * o * o * o * v * v * v;
            t3_assemble_m3_kernel<<<blocks_for(n), 256, 0, st>>>(o, v, Y, Z, Q12, Q13, eo, ev, t3);
        }
        CCSD_LAUNCH_CHECK();
        return;
    }
    if (V >= 3 && slab_smem_bytes(o, 3) <= kSlabSmemMax) {  // O <= 20
        opt_in_smem(t3_assemble_unique_kernel<false>, configured_unique);
        t3_assemble_unique_kernel<false><<<(unsigned)triples, 256, slab_smem_bytes(o, 3), st>>>(o, v, Y, Z, nullptr,
                                                                                              nullptr, eo, ev, t3);
        CCSD_LAUNCH_CHECK();
        return;
    }
    if (V >= 3 && slab_smem_bytes(o, 2) <= kSlabSmemMax) {  // O <= 24
        opt_in_smem(t3_assemble_slab_kernel, configured_slab);
        t3_assemble_slab_kernel<<<(unsigned)triples, 256, slab_smem_bytes(o, 2), st>>>(o, v, Y, Z, eo, ev, t3);
        CCSD_LAUNCH_CHECK();
        return;
    }
    // fewer than three virtual spin orbitals (t3 is zero) or O^3 slabs beyond shared memory
    const size_t n = (size_t)64 * o * o * o * v * v * v;
    t3_assemble_kernel<<<blocks_for(n), 256, 0, st>>>(o, v, Y, Z, eo, ev, t3);
    CCSD_LAUNCH_CHECK();
}

}  // namespace ccsd
