// Internal declarations shared by the host engine (C++) and the CUDA kernels.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>

struct ccsd_basis;  // include/ccsd_gb300.h

namespace ccsd {

// Status carried through the engine as an exception internally; converted to
// a C status code at the ABI boundary (abi.cpp).
struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

// An allocation that an update asked for while its launches were being captured
// into a CUDA graph (where cudaMalloc / cudaFree are not allowed): the capture is
// dropped and the update runs directly, which makes the allocation.
struct CaptureMiss : Error {
    explicit CaptureMiss(const std::string &m) : Error(-3, m) {}
};

#define CCSD_CUDA(call)                                                                    \
    do {                                                                                   \
        cudaError_t e_ = (call);                                                           \
        if (e_ != cudaSuccess) {                                                           \
            throw ::ccsd::Error(e_ == cudaErrorMemoryAllocation ? -3 : -2,                 \
                                std::string(#call) + ": " + cudaGetErrorString(e_) + " (" + \
                                    __FILE__ + ":" + std::to_string(__LINE__) + ")");      \
        }                                                                                  \
    } while (0)

// One logical matrix dimension made of up to three tensor sub-indices,
// outermost first: idx -> (i0, i1, i2) with i2 = idx % e2,
// i1 = (idx / e2) % e1, i0 = idx / (e1 * e2); offset = i0*s0 + i1*s1 + i2*s2.
// An unused level keeps the extent UINT32_MAX, so a 1-level dim is i2 = idx
// and a 2-level dim is (i1, i2).  This lets a GEMM read a 4-index tensor in
// any grouping without a copy.
// The divisions by e2 and e1 are multiply-highs with precomputed constants
// (Granlund & Montgomery 1994, the round-up form for 32-bit operands):
// n / e = (umulhi(m, n) + n) >> l with l = ceil(log2 e) and
// m = floor(2^32 (2^l - e) / e) + 1, exact for every 32-bit n.  A 1-level dim
// skips the divisions altogether; these offsets are computed per element in the
// splitter, the FP64 kernels and the epilogues.
struct Dim {
    uint32_t e1 = 0xFFFFFFFFu, e2 = 0xFFFFFFFFu;
    int64_t s0 = 0, s1 = 0, s2 = 0;
    uint32_t m1 = 0, m2 = 0, l1 = 0, l2 = 0;  // division constants for e1, e2
};

__host__ __device__ inline uint32_t dim_udiv(uint32_t n, uint32_t m, uint32_t l) {
#ifdef __CUDA_ARCH__
    const uint32_t t = __umulhi(m, n);
#else
    const uint32_t t = (uint32_t)(((uint64_t)m * n) >> 32);
#endif
    return (uint32_t)(((uint64_t)t + n) >> l);
}

__host__ __device__ inline int64_t dim_off(const Dim &d, uint32_t idx) {
    if (d.e2 == 0xFFFFFFFFu) return (int64_t)idx * d.s2;
    const uint32_t q = dim_udiv(idx, d.m2, d.l2), i2 = idx - q * d.e2;
    if (d.e1 == 0xFFFFFFFFu) return (int64_t)q * d.s1 + (int64_t)i2 * d.s2;
    const uint32_t i0 = dim_udiv(q, d.m1, d.l1), i1 = q - i0 * d.e1;
    return (int64_t)i0 * d.s0 + (int64_t)i1 * d.s1 + (int64_t)i2 * d.s2;
}

inline void dim_magic(uint32_t e, uint32_t &m, uint32_t &l) {
    m = l = 0;
    if (e == 0) return;  // an empty view: no index reaches the division
    uint32_t ll = 0;
    while (ll < 32 && (1ull << ll) < e) ++ll;
    l = ll;
    m = (uint32_t)((((uint64_t)1 << 32) * (((uint64_t)1 << ll) - e)) / e + 1);
}

// Helpers to build dims.
inline Dim ix1(int64_t s) { Dim d; d.s2 = s; return d; }
inline Dim ix2(uint32_t e_inner, int64_t s_outer, int64_t s_inner) {
    Dim d; d.e2 = e_inner; d.s1 = s_outer; d.s2 = s_inner;
    dim_magic(e_inner, d.m2, d.l2);
    return d;
}
inline Dim ix3(uint32_t e_mid, uint32_t e_inner, int64_t s_outer, int64_t s_mid, int64_t s_inner) {
    Dim d; d.e1 = e_mid; d.e2 = e_inner; d.s0 = s_outer; d.s1 = s_mid; d.s2 = s_inner;
    dim_magic(e_mid, d.m1, d.l1);
    dim_magic(e_inner, d.m2, d.l2);
    return d;
}

// A read-only matrix view rows x cols over a tensor.
struct MatView {
    const double *p = nullptr;
    Dim row, col;
};
// A writable matrix view.
struct OutView {
    double *p = nullptr;
    Dim row, col;
};

// Count of kernel launches issued by this library (host side, all threads).
void note_launch(int n = 1);
long launch_count();
// After every <<<...>>> launch: check it and count it.
#define CCSD_LAUNCH_CHECK()                 \
    do {                                    \
        CCSD_CUDA(cudaGetLastError());      \
        ::ccsd::note_launch();              \
    } while (0)

// ---- FP64 kernels (gemm_f64.cu, tensor_ops.cu) ------------------------------
// C(m,n) = alpha * sum_k A(m,k) * B(n,k) + beta * C(m,n); A is M x K, B is N x K.
// `ws` is scratch of `ws_elems` doubles used for split-K partial sums.
void gemm_f64(int M, int N, int K, double alpha, const MatView &A, const MatView &B, double beta,
              const OutView &C, double *ws, size_t ws_elems, cudaStream_t st);
// Elements needed in `ws` for this GEMM shape (0 when no split-K is used).
size_t gemm_f64_ws_elems(int M, int N, int K);

// Y(r,c) = alpha * X(r,c) + beta * Y(r,c) over an R x C grid (views may permute).
void axpby_view(int R, int C, double alpha, const MatView &X, double beta, const OutView &Y,
                cudaStream_t st);
// Y = alpha X + beta Yin, Yin read at Y's offsets (another array laid out like Y), by the
// permute form only; returns false (nothing launched) where that form does not apply
bool axpby_view_from(int R, int C, double alpha, const MatView &X, double beta, const double *Yin,
                     const OutView &Y, cudaStream_t st);

// Elementwise/amplitude kernels (all closed-shell spatial, o = nocc, v = nvir).
void k_tau(int o, int v, const double *t1, const double *t2, double *tau, cudaStream_t st);
// tau as k_tau, and the nblocks block partials of sum_n L[n] tau[n] in the same pass
void k_tau_dot(int o, int v, const double *t1, const double *t2, const double *L, double *tau, double *partials,
               int nblocks, cudaStream_t st);
void k_mp2_guess(int o, int v, const double *ovov, const double *eo, const double *ev, double *t2,
                 cudaStream_t st);
void k_theta(int o, int v, const double *t1, const double *t2, double *th1, double *th2,
             cudaStream_t st);
// t2_new = (R + Rp + Rp^T) / D2, returns into t2_new; also writes the per-block
// partial sums of |t2_new - t2_old|^2 into `partials` (length >= grid).
// Gaussian integrals of a basis (gto_ints.cu); device_out: S/T/V/eri are device pointers
void ao_integrals(const ::ccsd_basis &bs, double *S, double *T, double *V, double *eri, double *e_nuc,
                  bool device_out, cudaStream_t st);
// R[i][j][a][b] = R[j][i][b][a] = their mean (o o v v, in place)
void k_pair_mean(int o, int v, double *R, cudaStream_t st);
// dinv2 (o o v v: 1 / D_ij^ab, from k_dinv2) may be NULL: then D is formed and divided per element.
// partials NULL (dinv2 given): no partial sums of |t2_new - t2_old|^2, and t2_old is not read
void k_update_t2(int o, int v, const double *R, const double *Rp, const double *eo,
                 const double *ev, const double *dinv2, const double *t2_old, double *t2_new,
                 double *partials, int nblocks, cudaStream_t st);
void k_dinv2(int o, int v, const double *eo, const double *ev, double *dinv, cudaStream_t st);
// DIIS: one pass stores T_s = x_new and E_s = x_new - x_old (x = t1 then t2, lengths n1 + n2) and
// writes the block partials of <E_s, others[q]> (others[q] NULL: E_s itself) at partials[q * nblocks]
void k_diis_store(size_t n1, size_t n2, const double *x1n, const double *x2n, const double *x1o,
                  const double *x2o, double *Ts, double *Es, const double *const *others, int nothers,
                  double *partials, int nblocks, cudaStream_t st);
// (y1, y2) = sum_q coef[q] vecs[q] in one pass (n <= 16)
void k_diis_combine(size_t n1, size_t n2, const double *const *vecs, const double *coef, int n, double *y1,
                    double *y2, cudaStream_t st);
// y = a x1 + b x2 over n contiguous elements (16-byte aligned arrays)
void k_lincomb2(size_t n, double a, const double *x1, double b, const double *x2, double *y, cudaStream_t st);
// Foo[k][i] += sum_l (2 X[k][l][i][l] - X[k][l][l][i]) for X[k][l][i][j] (o^4)
void k_foo_from_x(int o, const double *X, double *Foo, cudaStream_t st);
// S[i][j][a][k] = tmpB[k][i][a][j] + Z[i][j][k][a] + Vk[k][j][a][i] (o^3 v each)
void k_t1_terms(int o, int v, const double *tmpB, const double *Z, const double *Vk, double *S, cudaStream_t st);
// out[a][c] += coef sum_k P[k sk + a sa + c sc] for a, c < v, k < o
void k_diag_acc(int o, int v, double coef, const double *P, int64_t sk, int64_t sa, int64_t sc, double *out,
                cudaStream_t st);
// R1[i][a] += sum_k (2 Z[i][k][k][a] - Z[k][i][k][a]) for Z[i][j][k][a] (o o o v)
void k_r1_from_z(int o, int v, const double *Z, double *R1, cudaStream_t st);
// out[q] = sum of partials[q * nparts .. q * nparts + nparts) for q < nq
void k_multi_sum(int nq, int nparts, const double *partials, double *out, cudaStream_t st);
void k_update_t1(int o, int v, const double *R1, const double *eo, const double *ev,
                 const double *t1_old, double *t1_new, double *partials, cudaStream_t st);
// E = sum_{ijab} L[i,j,a,b] * tau[i,j,a,b]; block partial sums into `partials`.
void k_dot(size_t n, const double *x, const double *y, double *partials, int nblocks,
           cudaStream_t st);
// sum of `n` partials into out[0] (single block, deterministic order).
void k_sum(int n, const double *partials, double *out, cudaStream_t st);
// Symmetric/antisymmetric particle-particle ladder (ladder_sym.cu); pair
// indices tri(p>=q) = p(p+1)/2 + q and stri(p>q) = p(p-1)/2 + q.
// tau+[tri(i,j)][tri(c,d)], tau-[stri(i,j)][stri(c,d)] from tau[i][j][c][d]
void k_tau_sym(int o, int v, const double *tau, double *tp, double *tm, cudaStream_t st);
void k_tau_sym_adj(int o, int v, const double *tpb, const double *tmb, double *taub, cudaStream_t st);
// R[i][j][a][b] += S+[tri(i,j)][tri(a,b)] + sgn(i-j) sgn(a-b) S-[stri(i,j)][stri(a,b)]
void k_ladder_unpack(int o, int v, const double *sp, const double *sm, double *R, cudaStream_t st);
void k_ladder_unpack_adj(int o, int v, const double *Rb, double *spb, double *smb, cudaStream_t st);
// W+[tri(a,b)][tri(c,d)], W-[stri(a,b)][stri(c,d)] from W[a][b][c][d] = (ac|bd)
void k_w_sym(int v, const double *W, double *wp, double *wm, cudaStream_t st);
void k_w_sym_adj(int v, const double *wpb, const double *wmb, double *Wb, cudaStream_t st);
// V+[(k,a)][tri(c,d)] = (kd|ac) + (kc|ad) (c > d), (kc|ac) (c = d); V-[(k,a)][stri(c,d)] =
// (kd|ac) - (kc|ad), from ovvv[k][d][a][c] = (kd|ac)
void k_ovvv_pair_pack(int o, int v, const double *ovvv, double *vp, double *vm, cudaStream_t st);
// Z[i][j][n] = Zs[tri(i,j)][n] + sgn(i-j) Za[stri(i,j)][n], n < o v (za may be null)
void k_z_pair_unpack(int o, int v, const double *zs, const double *za, double *Z, cudaStream_t st);
// U+[(k,l)][tri(c,d)] = (kc|ld) + (kd|lc) (c > d), (kc|lc) (c = d); U-[(k,l)][stri(c,d)] =
// (kc|ld) - (kd|lc), from ovov[k][c][l][d] = (kc|ld)
void k_ovov_pair_pack(int o, int v, const double *ovov, double *up, double *um, cudaStream_t st);
// X[r][i][j] = Xs[r][tri(i,j)] + sgn(i-j) Xa[r][stri(i,j)], r < o^2 (xa may be null)
void k_x_pair_unpack(int o, const double *xs, const double *xa, double *X, cudaStream_t st);
// W+[tri(i,j)][tri(k,l)] = W[kl,ij] + W[lk,ij] (k > l), W[kk,ij]; W-[stri(i,j)][stri(k,l)] =
// W[kl,ij] - W[lk,ij], from W[k][l][i][j]
void k_oooo_pair_pack(int o, const double *W, double *wp, double *wm, cudaStream_t st);
// CCSDT-1a triples (triples.cu), spin orbitals O = 2o, V = 2v:
// <PQ||RS> blocks from the spatial ovov/ovoo/ovvv blocks; kind 0: vvvo [b][c][e][k],
// 1: ovoo [m][c][j][k], 2: oovv [j][k][b][c], 3: vovv [b][k][c][d], 4: ooov [k][m][j][c],
// 5: voov [a][l][i][d], 6: oooo [m][l][i][j], 7: vvvv [a][b][e][d] (kinds 5-7 read oovv, oooo and
// wv[a][b][c][d] = (ac|bd); the others may pass them as NULL)
void k_so_block(int kind, int o, int v, const double *ovov, const double *ovoo, const double *ovvv,
                const double *oovv, const double *oooo, const double *wv, double *out, cudaStream_t st);
// tauso[a][b][i][j] = t2so + t1so[a][i] t1so[b][j] - t1so[a][j] t1so[b][i]
void k_tau_spin(int o, int v, const double *t2so, const double *t1so, double *tauso, cudaStream_t st);
// t1so[a][i] (spin orbitals) from the spatial t1[i][a]
void k_t1_spin(int o, int v, const double *t1, double *t1so, cudaStream_t st);
// t2so[a][b][i][j] (spin orbitals) from the spatial t2[i][j][a][b]
void k_t2_spin(int o, int v, const double *t2, double *t2so, cudaStream_t st);
// t3 = [P(a/bc) P(k/ij) Y - P(c/ab) P(i/jk) Z (+ P(i/jk) P(abc) Q12 + P(a/bc) P(ijk) Q13
// when Q12 is given)] / D3, all [a][b][c][i][j][k]
void k_t3_assemble(int o, int v, const double *Y, const double *Z, const double *Q12, const double *Q13,
                   const double *eo, const double *ev, double *t3, cudaStream_t st);
void k_fill(size_t n, double val, double *p, cudaStream_t st);
void k_copy_diag(int n, const double *fock, int off, int cnt, double *out, cudaStream_t st);
int reduce_blocks();

}  // namespace ccsd
