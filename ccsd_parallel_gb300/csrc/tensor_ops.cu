// Memory-bound kernels of the amplitude iteration: strided permute-add, tau,
// the T2/T1 energy-denominator updates, the MP2 guess and the deterministic
// reductions behind E_corr and the residual norm.  All FP64; their roofline
// is HBM bandwidth.
//
// Index conventions (closed-shell spatial): t1[i][a], t2[i][j][a][b].
#include <algorithm>
#include <atomic>

#include "common.h"
#include "fp64_ops.cuh"

namespace ccsd {

namespace {

constexpr int kReduceBlocks = 8 * 152;
constexpr int kReduceThreads = 256;

inline int grid_for(size_t n, int threads = 256) {
    size_t b = (n + threads - 1) / threads;
    if (b > 8 * 152 * 4) b = 8 * 152 * 4;
    if (b < 1) b = 1;
    return (int)b;
}

__global__ void axpby_view_kernel(int R, int C, double alpha, MatView X, double beta, OutView Y) {
    const int mode = axpby_mode(alpha, beta);
    const bool rx = axpby_reads_x(mode), ry = axpby_reads_y(mode);
    size_t total = (size_t)R * C;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
         idx += (size_t)gridDim.x * blockDim.x) {
        uint32_t r = (uint32_t)(idx / C), c = (uint32_t)(idx % C);
        double *y = Y.p + dim_off(Y.row, r) + dim_off(Y.col, c);
        const double x = rx ? X.p[dim_off(X.row, r) + dim_off(X.col, c)] : 0.0;
        *y = axpby_apply(mode, alpha, x, beta, ry ? *y : 0.0);
    }
}

// Y = alpha X + beta Y as a permutation over four indices (three row levels and
// the column) whose X strides and Y strides differ: a 32 x 32 tile over the
// index that is unit-stride in X (p) and the one unit-stride in Y (q) goes
// through shared memory, so that reads run along p and writes along q.  The
// other two indices and the tile numbers come from blockIdx.x.
struct PermIndex {
    uint32_t ext[4];
    int64_t xs[4], ys[4];
};
// the same with 32-bit strides, for views whose offsets all stay below 2^31 (64-bit
// integer multiplies and adds issue on the FP64 pipe on this part)
struct PermIndex32 {
    uint32_t ext[4];
    int32_t xs[4], ys[4];
};

// mode: axpby_mode(alpha, beta), classified on the host (a block here handles 4 elements
// per thread, so per-thread FP64 comparisons would cost more than the arithmetic)
// Yin: where the Y operand is read (Y itself, or another array with Y's offsets)
template <class PI, typename I>
__global__ void __launch_bounds__(256) permute_axpby_kernel(PI P, int p, int q, int u, int w, uint32_t tp,
                                                            uint32_t tq, int mode, double alpha,
                                                            const double *__restrict__ X, double beta,
                                                            const double *Yin, double *Y) {
    __shared__ double t[32][33];
    uint32_t b = blockIdx.x;
    const uint32_t ip0 = (b % tp) * 32;
    b /= tp;
    const uint32_t iq0 = (b % tq) * 32;
    b /= tq;
    const uint32_t iu = b % P.ext[u], iw = b / P.ext[u];
    const I xb = (I)iu * P.xs[u] + (I)iw * P.xs[w];
    const I yb = (I)iu * P.ys[u] + (I)iw * P.ys[w];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
    const bool ry = axpby_reads_y(mode);
    // this thread's Y elements are read before the exchange, so that the X and Y loads
    // are in flight together
    double yv[4];
#pragma unroll
    for (int j = 0; j < 32; j += 8) {
        const uint32_t iq = iq0 + tx, ip = ip0 + ty + j;
        yv[j / 8] = (ry && ip < P.ext[p] && iq < P.ext[q]) ? Yin[yb + (I)ip * P.ys[p] + (I)iq * P.ys[q]] : 0.0;
    }
#pragma unroll
    for (int j = 0; j < 32; j += 8) {
        const uint32_t ip = ip0 + tx, iq = iq0 + ty + j;
        double v = 0.0;
        if (ip < P.ext[p] && iq < P.ext[q]) v = X[xb + (I)ip * P.xs[p] + (I)iq * P.xs[q]];
        t[ty + j][tx] = v;
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < 32; j += 8) {
        const uint32_t iq = iq0 + tx, ip = ip0 + ty + j;
        if (ip < P.ext[p] && iq < P.ext[q])
            Y[yb + (I)ip * P.ys[p] + (I)iq * P.ys[q]] = axpby_apply(mode, alpha, t[tx][ty + j], beta, yv[j / 8]);
    }
}

// R * C < 2^32: 32-bit indices, and (r, c) = divmod(idx, C) as a multiply-high
// with the constants (cm, cl) of C (the same form as the view offsets)
// Four elements per thread and iteration (blockDim apart, so loads stay
// coalesced), their loads issued before any store.
__global__ void axpby_view32_kernel(int R, int C, uint32_t cm, uint32_t cl, double alpha, MatView X, double beta,
                                    OutView Y) {
    const uint32_t total = (uint32_t)R * (uint32_t)C;
    const uint32_t step = gridDim.x * blockDim.x * 4u;
    const int mode = axpby_mode(alpha, beta);
    const bool rx = axpby_reads_x(mode), ry = axpby_reads_y(mode);
    for (uint32_t base = blockIdx.x * blockDim.x * 4u + threadIdx.x; base < total; base += step) {
        double *yp[4];
        double xv[4], yv[4];
        bool in[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const uint32_t idx = base + u * blockDim.x;
            in[u] = idx < total && idx >= base;  // idx >= base: no 32-bit wrap
            const uint32_t r = dim_udiv(in[u] ? idx : 0u, cm, cl), c = (in[u] ? idx : 0u) - r * (uint32_t)C;
            yp[u] = Y.p + dim_off(Y.row, r) + dim_off(Y.col, c);
            xv[u] = (in[u] && rx) ? X.p[dim_off(X.row, r) + dim_off(X.col, c)] : 0.0;
            yv[u] = (in[u] && ry) ? *yp[u] : 0.0;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (in[u]) *yp[u] = axpby_apply(mode, alpha, xv[u], beta, yv[u]);
    }
}

// y = a x1 + b x2 over n contiguous elements, two doubles per load
__global__ void lincomb2_kernel(size_t n, double a, const double *__restrict__ x1, double b,
                                const double *__restrict__ x2, double *__restrict__ y) {
    const size_t n2 = n / 2;
    const double2 *p1 = reinterpret_cast<const double2 *>(x1), *p2 = reinterpret_cast<const double2 *>(x2);
    double2 *q = reinterpret_cast<double2 *>(y);
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n2; i += (size_t)gridDim.x * blockDim.x) {
        const double2 u = p1[i], w = p2[i];
        q[i] = make_double2(fma(b, w.x, a * u.x), fma(b, w.y, a * u.y));
    }
    if (blockIdx.x == 0 && threadIdx.x == 0 && (n & 1)) y[n - 1] = fma(b, x2[n - 1], a * x1[n - 1]);
}

__global__ void tau_kernel(int o, int v, const double *t1, const double *t2, double *tau) {
    size_t total = (size_t)o * o * v * v;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
         idx += (size_t)gridDim.x * blockDim.x) {
        int b = idx % v;
        size_t r = idx / v;
        int a = r % v;
        r /= v;
        int j = r % o;
        int i = (int)(r / o);
        tau[idx] = t2[idx] + t1[i * v + a] * t1[j * v + b];
    }
}

// th1[i,a,l,d] = t2[i,l,a,d] - t2[i,l,d,a]/2 - t1[i,d] t1[l,a]
// th2[i,a,l,d] = t2[i,l,d,a]/2 + t1[i,d] t1[l,a]
__global__ void theta_kernel(int o, int v, const double *t1, const double *t2, double *th1,
                             double *th2) {
    size_t total = (size_t)o * v * o * v;
    size_t ov2 = (size_t)o * v * v, v2 = (size_t)v * v;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
         idx += (size_t)gridDim.x * blockDim.x) {
        int d = idx % v;
        size_t r = idx / v;
        int l = r % o;
        r /= o;
        int a = r % v;
        int i = (int)(r / v);
        double tad = t2[i * ov2 + l * v2 + (size_t)a * v + d];
        double tda = t2[i * ov2 + l * v2 + (size_t)d * v + a];
        double tt = t1[i * v + d] * t1[l * v + a];
        const double h = fma(0.5, tda, tt);
        th1[idx] = tad - h;
        th2[idx] = h;
    }
}

__global__ void mp2_kernel(int o, int v, const double *ovov, const double *eo, const double *ev,
                           double *t2) {
    size_t total = (size_t)o * o * v * v;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
         idx += (size_t)gridDim.x * blockDim.x) {
        int b = idx % v;
        size_t r = idx / v;
        int a = r % v;
        r /= v;
        int j = r % o;
        int i = (int)(r / o);
        double g = ovov[(((size_t)i * v + a) * o + j) * v + b];
        t2[idx] = g / (eo[i] + eo[j] - ev[a] - ev[b]);
    }
}

__device__ double block_sum(double x) {
    __shared__ double sh[32];
    for (int off = 16; off > 0; off >>= 1) x += __shfl_down_sync(0xffffffffu, x, off);
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) sh[w] = x;
    __syncthreads();
    double s = 0.0;
    if (w == 0) {
        int nw = blockDim.x >> 5;
        s = lane < nw ? sh[lane] : 0.0;
        for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
    }
    __syncthreads();
    return s;  // valid in thread 0
}

__global__ void update_t2_kernel(int o, int v, const double *R, const double *Rp,
                                 const double *eo, const double *ev, const double *t2_old,
                                 double *t2_new, double *partials) {
    size_t total = (size_t)o * o * v * v;
    size_t v2 = (size_t)v * v, ov2 = (size_t)o * v2;
    double acc = 0.0;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
         idx += (size_t)gridDim.x * blockDim.x) {
        int b = idx % v;
        size_t r = idx / v;
        int a = r % v;
        r /= v;
        int j = r % o;
        int i = (int)(r / o);
        double num = R[idx] + Rp[idx] + Rp[j * ov2 + i * v2 + (size_t)b * v + a];
        double t = num / (eo[i] + eo[j] - ev[a] - ev[b]);
        double d = t - t2_old[idx];
        acc = fma(d, d, acc);
        t2_new[idx] = t;
    }
    double s = block_sum(acc);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

// R[i][j][a][b] and R[j][i][b][a] both become their mean; the thread at the
// smaller index of a pair does both writes
__global__ void pair_mean_kernel(int o, int v, double *R) {
    const size_t total = (size_t)o * o * v * v, v2 = (size_t)v * v, ov2 = (size_t)o * v2;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
         idx += (size_t)gridDim.x * blockDim.x) {
        const int b = (int)(idx % v);
        size_t r = idx / v;
        const int a = (int)(r % v);
        r /= v;
        const int j = (int)(r % o), i = (int)(r / o);
        const size_t p = (size_t)j * ov2 + (size_t)i * v2 + (size_t)b * v + a;
        if (p <= idx) continue;
        const double m = 0.5 * (R[idx] + R[p]);
        R[idx] = m;
        R[p] = m;
    }
}

// ---- 32 x 32 tiles over the (a, b) indices of an o x o x v x v array ---------
// A block (32 x 8 threads) walks tiles t = ((i o + j) nt + A) nt + B, nt = ceil(v/32);
// tile indices are decoded once per tile, never per element.  Element (a, b) of a
// tile is a = 32 A + q (q = ty, ty + 8, ...), b = 32 B + tx, so global loads and
// stores along b are coalesced; a partner read with a and b exchanged goes through
// a shared-memory tile loaded along its own contiguous index.
struct Tile4 {
    int i, j, A, B;
};
__device__ __forceinline__ Tile4 tile_of(int t, int o, int nt) {
    Tile4 T;
    T.B = t % nt;
    t /= nt;
    T.A = t % nt;
    t /= nt;
    T.j = t % o;
    T.i = t / o;
    return T;
}

// 1 / (eo[i] + eo[j] - ev[a] - ev[b]) over [i][j][a][b] (fixed for a solve)
__global__ void dinv2_kernel(int o, int v, const double *eo, const double *ev, double *dinv) {
    const int rows = o * o * v;
    for (int r = blockIdx.x; r < rows; r += gridDim.x) {
        const int a = r % v, ij = r / v, j = ij % o, i = ij / o;
        const double dij = eo[i] + eo[j] - ev[a];
        for (int b = threadIdx.x; b < v; b += blockDim.x) dinv[(size_t)r * v + b] = 1.0 / (dij - ev[b]);
    }
}

// t2_new = (R + Rp + Rp^T) * dinv with Rp^T[i][j][a][b] = Rp[j][i][b][a]; per-block
// partial sums of |t2_new - t2_old|^2 (a fixed tile order per block: deterministic)
// NORM = false: no partial sums (the caller takes the norm elsewhere) and t2o is not read
// I: the index type, int32_t when every offset is below 2^31 (64-bit integer arithmetic
// issues on the FP64 pipe on this part), else int64_t
template <bool NORM, typename I>
__global__ void __launch_bounds__(256) update_t2_tiled_kernel(int o, int v, const double *__restrict__ R,
                                                              const double *__restrict__ Rp,
                                                              const double *__restrict__ dinv,
                                                              const double *__restrict__ t2o,
                                                              double *__restrict__ t2n, double *partials) {
    __shared__ double s[32][33];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int nt = (v + 31) / 32, ntiles = o * o * nt * nt;
    const I v2 = (I)v * v;
    double acc = 0.0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const Tile4 T = tile_of(t, o, nt);
        const double *rpt = Rp + ((I)T.j * o + T.i) * v2;  // Rp[j][i][b][a], read along a
        for (int q = ty; q < 32; q += 8) {
            const int b = T.B * 32 + q, a = T.A * 32 + tx;
            s[q][tx] = (b < v && a < v) ? rpt[(I)b * v + a] : 0.0;
        }
        __syncthreads();
        const I base = ((I)T.i * o + T.j) * v2;
        const int b = T.B * 32 + tx;
        for (int q = ty; q < 32; q += 8) {
            const int a = T.A * 32 + q;
            if (a < v && b < v) {
                const I idx = base + (I)a * v + b;
                const double tn = (R[idx] + Rp[idx] + s[tx][q]) * dinv[idx];
                if (NORM) {
                    const double d = tn - t2o[idx];
                    acc = fma(d, d, acc);
                }
                t2n[idx] = tn;
            }
        }
        __syncthreads();
    }
    if (NORM) {
        const double sum = block_sum(acc);
        if (threadIdx.x == 0) partials[blockIdx.x] = sum;
    }
}

// th1[i,a,l,d] = t2[i,l,a,d] - t2[i,l,d,a]/2 - t1[i,d] t1[l,a]; th2[i,a,l,d] = t2[i,l,d,a]/2 + t1[i,d] t1[l,a]
// (tiles over (a, d) for each (i, l))
template <typename I>
__global__ void __launch_bounds__(256) theta_tiled_kernel(int o, int v, const double *__restrict__ t1,
                                                          const double *__restrict__ t2, double *__restrict__ th1,
                                                          double *__restrict__ th2) {
    __shared__ double s[32][33];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int nt = (v + 31) / 32, ntiles = o * o * nt * nt;
    const I v2 = (I)v * v;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const Tile4 T = tile_of(t, o, nt);  // (i, l, A, D)
        const int i = T.i, l = T.j;
        const double *t2il = t2 + ((I)i * o + l) * v2;
        for (int q = ty; q < 32; q += 8) {  // s[d][a] = t2[i,l,d,a]
            const int d = T.B * 32 + q, a = T.A * 32 + tx;
            s[q][tx] = (d < v && a < v) ? t2il[(I)d * v + a] : 0.0;
        }
        __syncthreads();
        const int d = T.B * 32 + tx;
        for (int q = ty; q < 32; q += 8) {
            const int a = T.A * 32 + q;
            if (a < v && d < v) {
                const double tad = t2il[(I)a * v + d];
                const double tda = s[tx][q];
                const double tt = t1[i * v + d] * t1[l * v + a];
                const I out = (((I)i * v + a) * o + l) * v + d;
                const double h = fma(0.5, tda, tt);  // th1 + th2 = t2[i,l,a,d]: three FP64 operations
                th1[out] = tad - h;
                th2[out] = h;
            }
        }
        __syncthreads();
    }
}

// tau[i][j][a][b] = t2 + t1[i][a] t1[j][b], one row (i, j, a) at a time
__global__ void tau_rows_kernel(int o, int v, const double *__restrict__ t1, const double *__restrict__ t2,
                                double *__restrict__ tau) {
    const int rows = o * o * v;
    for (int r = blockIdx.x; r < rows; r += gridDim.x) {
        const int a = r % v, ij = r / v, j = ij % o, i = ij / o;
        const double ta = t1[i * v + a];
        const double *t1j = t1 + (size_t)j * v;
        const size_t base = (size_t)r * v;
        for (int b = threadIdx.x; b < v; b += blockDim.x) tau[base + b] = t2[base + b] + ta * t1j[b];
    }
}

// ---- DIIS on the amplitude vector x = (t1, t2) ---------------------------------
// store: T_s = x_new, E_s = x_new - x_old, and the block partials of <E_s, E_j>
// for the listed slots j (E_s itself included), all in one pass.
constexpr int kDiisMax = 16;
struct DiisVecs {
    const double *p[kDiisMax];
    double c[kDiisMax];
    int n;
};

// I: the index type (int32_t below 2^31 elements: 64-bit integer arithmetic issues on
// the FP64 pipe on this part)
template <typename I>
__global__ void __launch_bounds__(256) diis_store_kernel(I n1, I n2, const double *__restrict__ x1n,
                                                         const double *__restrict__ x2n,
                                                         const double *__restrict__ x1o,
                                                         const double *__restrict__ x2o, double *__restrict__ Ts,
                                                         double *__restrict__ Es, DiisVecs others,
                                                         double *partials) {
    double acc[kDiisMax];
#pragma unroll
    for (int q = 0; q < kDiisMax; ++q) acc[q] = 0.0;
    const I n = n1 + n2;
    for (I idx = blockIdx.x * (I)blockDim.x + threadIdx.x; idx < n; idx += (I)gridDim.x * blockDim.x) {
        const double xn = idx < n1 ? x1n[idx] : x2n[idx - n1];
        const double xo = idx < n1 ? x1o[idx] : x2o[idx - n1];
        const double e = xn - xo;
        Ts[idx] = xn;
        Es[idx] = e;
#pragma unroll
        for (int q = 0; q < kDiisMax; ++q)
            if (q < others.n) acc[q] = fma(e, others.p[q] ? others.p[q][idx] : e, acc[q]);
    }
    for (int q = 0; q < others.n; ++q) {
        const double sum = block_sum(acc[q]);
        if (threadIdx.x == 0) partials[(size_t)q * gridDim.x + blockIdx.x] = sum;
    }
}

// extrapolate: (y1, y2) = sum_q c_q V_q, V_q = (t1 part of length n1, t2 part); NV
// vectors, all loads of an element issued together
template <int NV, typename I>
__global__ void __launch_bounds__(256) diis_combine_kernel(I n1, I n2, DiisVecs vecs,
                                                           double *__restrict__ y1, double *__restrict__ y2) {
    const I n = n1 + n2;
    for (I idx = blockIdx.x * (I)blockDim.x + threadIdx.x; idx < n; idx += (I)gridDim.x * blockDim.x) {
        double x[NV];
#pragma unroll
        for (int q = 0; q < NV; ++q) x[q] = __ldcs(vecs.p[q] + idx);
        double s = 0.0;
#pragma unroll
        for (int q = 0; q < NV; ++q) s = fma(vecs.c[q], x[q], s);
        if (idx < n1)
            y1[idx] = s;
        else
            y2[idx - n1] = s;
    }
}

// R1[i][a] += sum_k (2 Z[i][k][k][a] - Z[k][i][k][a]),  Z[i][j][k][a] = sum_cd (kd|ac) tau[i,j,c,d]
__global__ void r1_from_z_kernel(int o, int v, const double *__restrict__ Z, double *__restrict__ R1) {
    const int n = o * v;
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x) {
        const int i = idx / v, a = idx % v;
        double s = 0.0;
        for (int k = 0; k < o; ++k) {
            const double zd = Z[(((size_t)i * o + k) * o + k) * v + a];
            const double zx = Z[(((size_t)k * o + i) * o + k) * v + a];
            s += 2.0 * zd - zx;
        }
        R1[idx] += s;
    }
}

// out[a][c] += coef sum_k P[k sk + a sa + c sc] over a v x v output (a diagonal of a
// larger product, summed over its repeated index k)
__global__ void diag_acc_kernel(int o, int v, double coef, const double *__restrict__ P, int64_t sk, int64_t sa,
                                int64_t sc, double *__restrict__ out) {
    const int n = v * v;
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x) {
        const int a = idx / v, c = idx % v;
        const double *q = P + a * sa + c * sc;
        double s = 0.0;
        for (int k = 0; k < o; ++k) s += q[k * sk];
        out[idx] += coef * s;
    }
}

// S[i][j][a][k] = tmpB[k][i][a][j] + Z[i][j][k][a] + Vk[k][j][a][i] (all o^3 v); a thread
// per (i, j, a, k), k fastest (the writes run along memory; the operands are 33 MB at o = 24, v = 300)
__global__ void t1_terms_kernel(int o, int v, const double *__restrict__ tmpB, const double *__restrict__ Z,
                                const double *__restrict__ Vk, double *__restrict__ S) {
    const size_t n = (size_t)o * o * v * o;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < n; idx += (size_t)gridDim.x * blockDim.x) {
        const int k = (int)(idx % o);
        size_t r = idx / o;
        const int a = (int)(r % v);
        r /= v;
        const int j = (int)(r % o), i = (int)(r / o);
        const double t = tmpB[(((size_t)k * o + i) * v + a) * o + j];
        const double z = Z[(((size_t)i * o + j) * o + k) * v + a];
        const double w = Vk[(((size_t)k * o + j) * v + a) * o + i];
        S[idx] = (t + z) + w;
    }
}

// Foo[k][i] += sum_l (2 X[k][l][i][l] - X[k][l][l][i])
__global__ void foo_from_x_kernel(int o, const double *__restrict__ X, double *__restrict__ Foo) {
    const int n = o * o;
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x) {
        const int k = idx / o, i = idx % o;
        double s = 0.0;
        for (int l = 0; l < o; ++l) {
            const size_t kl = ((size_t)k * o + l) * o;
            s += 2.0 * X[(kl + i) * o + l] - X[(kl + l) * o + i];
        }
        Foo[idx] += s;
    }
}

// sums of `nq` groups of `nparts` partials: out[q] = sum_b partials[q * nparts + b]
__global__ void multi_sum_kernel(int nq, int nparts, const double *partials, double *out) {
    for (int q = 0; q < nq; ++q) {
        double acc = 0.0;
        for (int i = threadIdx.x; i < nparts; i += blockDim.x) acc += partials[(size_t)q * nparts + i];
        const double s = block_sum(acc);
        if (threadIdx.x == 0) out[q] = s;
    }
}

__global__ void update_t1_kernel(int o, int v, const double *R1, const double *eo,
                                 const double *ev, const double *t1_old, double *t1_new,
                                 double *partials) {
    double acc = 0.0;
    for (int idx = threadIdx.x; idx < o * v; idx += blockDim.x) {
        int i = idx / v, a = idx % v;
        double t = R1[idx] / (eo[i] - ev[a]);
        double d = t - t1_old[idx];
        acc = fma(d, d, acc);
        t1_new[idx] = t;
    }
    double s = block_sum(acc);
    if (threadIdx.x == 0) partials[0] = s;
}

// tau = t2 + t1[i][a] t1[j][b] (as tau_rows_kernel) and the block partials of
// sum L tau in the same pass: a block takes rows (i, j, a) blockIdx.x, + gridDim.x, ...
__global__ void tau_dot_rows_kernel(int o, int v, const double *__restrict__ t1, const double *__restrict__ t2,
                                    const double *__restrict__ L, double *__restrict__ tau, double *partials) {
    const int rows = o * o * v;
    double acc = 0.0;
    for (int r = blockIdx.x; r < rows; r += gridDim.x) {
        const int a = r % v, ij = r / v, j = ij % o, i = ij / o;
        const double ta = t1[i * v + a];
        const double *t1j = t1 + j * v;
        const int base = r * v;  // o^2 v^2 < 2^31 (checked by the caller)
        for (int b = threadIdx.x; b < v; b += blockDim.x) {
            const double x = fma(ta, t1j[b], t2[base + b]);
            tau[base + b] = x;
            acc = fma(L[base + b], x, acc);
        }
    }
    const double s = block_sum(acc);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

__global__ void dot_kernel(size_t n, const double *x, const double *y, double *partials) {
    double acc = 0.0;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < n;
         idx += (size_t)gridDim.x * blockDim.x)
        acc = fma(x[idx], y[idx], acc);
    double s = block_sum(acc);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

__global__ void sum_kernel(int n, const double *partials, double *out) {
    double acc = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) acc += partials[i];
    double s = block_sum(acc);
    if (threadIdx.x == 0) out[0] = s;
}

__global__ void fill_kernel(size_t n, double val, double *p) {
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < n;
         idx += (size_t)gridDim.x * blockDim.x)
        p[idx] = val;
}

__global__ void copy_diag_kernel(int n, const double *fock, int off, int cnt, double *out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < cnt) out[i] = fock[(size_t)(off + i) * n + off + i];
}

}  // namespace

int reduce_blocks() { return kReduceBlocks; }

namespace {
std::atomic<long> g_launches{0};
}
void note_launch(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
long launch_count() { return g_launches.load(std::memory_order_relaxed); }

namespace {
// Row levels (outer, middle, inner) of a view over R rows: extents and strides.
bool row_levels(int R, const Dim &d, uint32_t ext[3], int64_t str[3]) {
    if (d.e2 == 0xFFFFFFFFu) {
        ext[0] = 1; ext[1] = 1; ext[2] = (uint32_t)R;
        str[0] = 0; str[1] = 0; str[2] = d.s2;
        return true;
    }
    if (d.e1 == 0xFFFFFFFFu) {
        if (R % d.e2) return false;
        ext[0] = 1; ext[1] = (uint32_t)(R / d.e2); ext[2] = d.e2;
        str[0] = 0; str[1] = d.s1; str[2] = d.s2;
        return true;
    }
    const uint64_t inner = (uint64_t)d.e1 * d.e2;
    if (R % inner) return false;
    ext[0] = (uint32_t)(R / inner); ext[1] = d.e1; ext[2] = d.e2;
    str[0] = d.s0; str[1] = d.s1; str[2] = d.s2;
    return true;
}

// The permute form when both views are plain 4-index views with the same row
// levels and 1-level columns, and their unit-stride indices differ.
bool try_permute_axpby(int R, int C, double alpha, const MatView &X, double beta, const OutView &Y, cudaStream_t st,
                       const double *Yin = nullptr) {
    if (!Yin) Yin = Y.p;
    if (X.col.e2 != 0xFFFFFFFFu || Y.col.e2 != 0xFFFFFFFFu) return false;
    if (X.row.e1 != Y.row.e1 || X.row.e2 != Y.row.e2) return false;
    PermIndex P;
    int64_t xr[3], yr[3];
    uint32_t ex[3], ey[3];
    if (!row_levels(R, X.row, ex, xr) || !row_levels(R, Y.row, ey, yr)) return false;
    for (int i = 0; i < 3; ++i) {
        P.ext[i] = ex[i];
        P.xs[i] = xr[i];
        P.ys[i] = yr[i];
    }
    P.ext[3] = (uint32_t)C;
    P.xs[3] = X.col.s2;
    P.ys[3] = Y.col.s2;
    int p = -1, q = -1;
    for (int i = 0; i < 4; ++i) {
        if (P.ext[i] > 1 && P.xs[i] == 1 && p < 0) p = i;
        if (P.ext[i] > 1 && P.ys[i] == 1 && q < 0) q = i;
    }
    if (p < 0 || q < 0 || p == q || P.ext[p] < 8 || P.ext[q] < 8) return false;
    int rest[2], nr = 0;
    for (int i = 0; i < 4; ++i)
        if (i != p && i != q) rest[nr++] = i;
    const uint32_t tp = (P.ext[p] + 31) / 32, tq = (P.ext[q] + 31) / 32;
    const uint64_t blocks = (uint64_t)tp * tq * P.ext[rest[0]] * P.ext[rest[1]];
    if (blocks >= (1ull << 31)) return false;
    int64_t xmax = 0, ymax = 0;  // largest offsets (strides here are non-negative)
    bool nonneg = true;
    for (int i = 0; i < 4; ++i) {
        nonneg = nonneg && P.xs[i] >= 0 && P.ys[i] >= 0;
        xmax += (int64_t)(P.ext[i] - 1) * P.xs[i];
        ymax += (int64_t)(P.ext[i] - 1) * P.ys[i];
    }
    if (nonneg && xmax < (1LL << 31) && ymax < (1LL << 31)) {
        PermIndex32 P32;
        for (int i = 0; i < 4; ++i) {
            P32.ext[i] = P.ext[i];
            P32.xs[i] = (int32_t)P.xs[i];
            P32.ys[i] = (int32_t)P.ys[i];
        }
        permute_axpby_kernel<PermIndex32, int32_t><<<(unsigned)blocks, 256, 0, st>>>(
            P32, p, q, rest[0], rest[1], tp, tq, axpby_mode(alpha, beta), alpha, X.p, beta, Yin, Y.p);
    } else {
        permute_axpby_kernel<PermIndex, int64_t><<<(unsigned)blocks, 256, 0, st>>>(
            P, p, q, rest[0], rest[1], tp, tq, axpby_mode(alpha, beta), alpha, X.p, beta, Yin, Y.p);
    }
    CCSD_LAUNCH_CHECK();
    return true;
}
}  // namespace

bool axpby_view_from(int R, int C, double alpha, const MatView &X, double beta, const double *Yin,
                     const OutView &Y, cudaStream_t st) {
    if (R <= 0 || C <= 0) return true;
    return try_permute_axpby(R, C, alpha, X, beta, Y, st, Yin);
}

void axpby_view(int R, int C, double alpha, const MatView &X, double beta, const OutView &Y,
                cudaStream_t st) {
    if (R <= 0 || C <= 0) return;
    if (try_permute_axpby(R, C, alpha, X, beta, Y, st)) return;
    if ((size_t)R * C < ((size_t)1 << 32) - ((size_t)1 << 22)) {  // idx + grid stride stays below 2^32
        uint32_t cm, cl;
        dim_magic((uint32_t)C, cm, cl);
        axpby_view32_kernel<<<grid_for((size_t)R * C), 256, 0, st>>>(R, C, cm, cl, alpha, X, beta, Y);
    } else {
        axpby_view_kernel<<<grid_for((size_t)R * C), 256, 0, st>>>(R, C, alpha, X, beta, Y);
    }
    CCSD_LAUNCH_CHECK();
}

// grids of the row and tile kernels: whole waves of 152 SMs
inline int rows_grid(long rows) { return (int)std::max(1L, std::min(rows, 152L * 16)); }
inline int tiles_grid(int o, int v) {
    const long nt = (v + 31) / 32, tiles = (long)o * o * nt * nt;
    return (int)std::max(1L, std::min(tiles, 152L * 8));
}

void k_tau(int o, int v, const double *t1, const double *t2, double *tau, cudaStream_t st) {
    if ((size_t)o * o * v * v >= ((size_t)1 << 31)) {  // row indices stay 32-bit in the row kernel
        tau_kernel<<<grid_for((size_t)o * o * v * v), 256, 0, st>>>(o, v, t1, t2, tau);
    } else {
        tau_rows_kernel<<<rows_grid((long)o * o * v), v <= 128 ? 128 : 320, 0, st>>>(o, v, t1, t2, tau);
    }
    CCSD_LAUNCH_CHECK();
}

void k_tau_dot(int o, int v, const double *t1, const double *t2, const double *L, double *tau, double *partials,
               int nblocks, cudaStream_t st) {
    if ((size_t)o * o * v * v >= ((size_t)1 << 31)) {
        k_tau(o, v, t1, t2, tau, st);
        k_dot((size_t)o * o * v * v, L, tau, partials, nblocks, st);
        return;
    }
    tau_dot_rows_kernel<<<nblocks, v <= 128 ? 128 : 320, 0, st>>>(o, v, t1, t2, L, tau, partials);
    CCSD_LAUNCH_CHECK();
}

void k_theta(int o, int v, const double *t1, const double *t2, double *th1, double *th2,
             cudaStream_t st) {
    if ((size_t)o * o * v * v >= ((size_t)1 << 31)) {
        theta_kernel<<<grid_for((size_t)o * o * v * v), 256, 0, st>>>(o, v, t1, t2, th1, th2);
    } else {
        theta_tiled_kernel<int32_t><<<tiles_grid(o, v), 256, 0, st>>>(o, v, t1, t2, th1, th2);  // o^2 v^2 < 2^31
    }
    CCSD_LAUNCH_CHECK();
}

void k_dinv2(int o, int v, const double *eo, const double *ev, double *dinv, cudaStream_t st) {
    dinv2_kernel<<<rows_grid((long)o * o * v), v <= 128 ? 128 : 320, 0, st>>>(o, v, eo, ev, dinv);
    CCSD_LAUNCH_CHECK();
}

void k_diis_store(size_t n1, size_t n2, const double *x1n, const double *x2n, const double *x1o,
                  const double *x2o, double *Ts, double *Es, const double *const *others, int nothers,
                  double *partials, int nblocks, cudaStream_t st) {
    if (nothers > kDiisMax) throw Error(-1, "DIIS: at most 16 vectors");
    DiisVecs d{};
    for (int q = 0; q < nothers; ++q) d.p[q] = others[q];
    d.n = nothers;
    if (n1 + n2 + (size_t)nblocks * 256 < ((size_t)1 << 31))
        diis_store_kernel<int32_t><<<nblocks, 256, 0, st>>>((int32_t)n1, (int32_t)n2, x1n, x2n, x1o, x2o, Ts, Es, d,
                                                            partials);
    else
        diis_store_kernel<int64_t><<<nblocks, 256, 0, st>>>((int64_t)n1, (int64_t)n2, x1n, x2n, x1o, x2o, Ts, Es, d,
                                                            partials);
    CCSD_LAUNCH_CHECK();
}

void k_diis_combine(size_t n1, size_t n2, const double *const *vecs, const double *coef, int n, double *y1,
                    double *y2, cudaStream_t st) {
    if (n > kDiisMax || n < 1) throw Error(-1, "DIIS: 1 to 16 vectors");
    DiisVecs d{};
    for (int q = 0; q < n; ++q) {
        d.p[q] = vecs[q];
        d.c[q] = coef[q];
    }
    d.n = n;
    const int g = (int)std::min<size_t>((n1 + n2 + 255) / 256, 152 * 8);
    const bool i32 = n1 + n2 + (size_t)g * 256 < ((size_t)1 << 31);
    switch (n) {
#define CCSD_DIIS_CASE(NV_)                                                                                 \
    case NV_:                                                                                               \
        if (i32)                                                                                            \
            diis_combine_kernel<NV_, int32_t><<<g, 256, 0, st>>>((int32_t)n1, (int32_t)n2, d, y1, y2);   \
        else                                                                                                \
            diis_combine_kernel<NV_, int64_t><<<g, 256, 0, st>>>((int64_t)n1, (int64_t)n2, d, y1, y2);   \
        break;
        CCSD_DIIS_CASE(1) CCSD_DIIS_CASE(2) CCSD_DIIS_CASE(3) CCSD_DIIS_CASE(4) CCSD_DIIS_CASE(5)
        CCSD_DIIS_CASE(6) CCSD_DIIS_CASE(7) CCSD_DIIS_CASE(8) CCSD_DIIS_CASE(9) CCSD_DIIS_CASE(10)
        CCSD_DIIS_CASE(11) CCSD_DIIS_CASE(12) CCSD_DIIS_CASE(13) CCSD_DIIS_CASE(14) CCSD_DIIS_CASE(15)
        CCSD_DIIS_CASE(16)
#undef CCSD_DIIS_CASE
    }
    CCSD_LAUNCH_CHECK();
}

void k_lincomb2(size_t n, double a, const double *x1, double b, const double *x2, double *y, cudaStream_t st) {
    if (n == 0) return;
    if (((uintptr_t)x1 | (uintptr_t)x2 | (uintptr_t)y) & 15)
        throw Error(-1, "lincomb2: operands must be 16-byte aligned");
    lincomb2_kernel<<<(int)std::min<size_t>((n / 2 + 255) / 256 + 1, 152 * 16), 256, 0, st>>>(n, a, x1, b, x2, y);
    CCSD_LAUNCH_CHECK();
}

void k_foo_from_x(int o, const double *X, double *Foo, cudaStream_t st) {
    foo_from_x_kernel<<<(o * o + 255) / 256, 256, 0, st>>>(o, X, Foo);
    CCSD_LAUNCH_CHECK();
}

void k_diag_acc(int o, int v, double coef, const double *P, int64_t sk, int64_t sa, int64_t sc, double *out,
                cudaStream_t st) {
    diag_acc_kernel<<<(v * v + 255) / 256, 256, 0, st>>>(o, v, coef, P, sk, sa, sc, out);
    CCSD_LAUNCH_CHECK();
}

void k_t1_terms(int o, int v, const double *tmpB, const double *Z, const double *Vk, double *S, cudaStream_t st) {
    t1_terms_kernel<<<grid_for((size_t)o * o * v * o), 256, 0, st>>>(o, v, tmpB, Z, Vk, S);
    CCSD_LAUNCH_CHECK();
}

void k_r1_from_z(int o, int v, const double *Z, double *R1, cudaStream_t st) {
    r1_from_z_kernel<<<(o * v + 255) / 256, 256, 0, st>>>(o, v, Z, R1);
    CCSD_LAUNCH_CHECK();
}

void k_multi_sum(int nq, int nparts, const double *partials, double *out, cudaStream_t st) {
    multi_sum_kernel<<<1, 1024, 0, st>>>(nq, nparts, partials, out);
    CCSD_LAUNCH_CHECK();
}

void k_mp2_guess(int o, int v, const double *ovov, const double *eo, const double *ev, double *t2,
                 cudaStream_t st) {
    mp2_kernel<<<grid_for((size_t)o * o * v * v), 256, 0, st>>>(o, v, ovov, eo, ev, t2);
    CCSD_LAUNCH_CHECK();
}

void k_update_t2(int o, int v, const double *R, const double *Rp, const double *eo,
                 const double *ev, const double *dinv2, const double *t2_old, double *t2_new,
                 double *partials, int nblocks, cudaStream_t st) {
    if (dinv2 && (size_t)o * o * v * v < ((size_t)1 << 31)) {
        if (partials)
            update_t2_tiled_kernel<true, int32_t><<<nblocks, 256, 0, st>>>(o, v, R, Rp, dinv2, t2_old, t2_new, partials);
        else
            update_t2_tiled_kernel<false, int32_t><<<nblocks, 256, 0, st>>>(o, v, R, Rp, dinv2, t2_old, t2_new, partials);
    } else if (!partials) {
        throw Error(-1, "k_update_t2: the norm-free form needs the 1/D table");
    } else
        update_t2_kernel<<<nblocks, kReduceThreads, 0, st>>>(o, v, R, Rp, eo, ev, t2_old, t2_new, partials);
    CCSD_LAUNCH_CHECK();
}

void k_pair_mean(int o, int v, double *R, cudaStream_t st) {
    const size_t n = (size_t)o * o * v * v;
    if (n == 0) return;
    pair_mean_kernel<<<grid_for(n), 256, 0, st>>>(o, v, R);
    CCSD_LAUNCH_CHECK();
}

void k_update_t1(int o, int v, const double *R1, const double *eo, const double *ev,
                 const double *t1_old, double *t1_new, double *partials, cudaStream_t st) {
    update_t1_kernel<<<1, 1024, 0, st>>>(o, v, R1, eo, ev, t1_old, t1_new, partials);
    CCSD_LAUNCH_CHECK();
}

void k_dot(size_t n, const double *x, const double *y, double *partials, int nblocks,
           cudaStream_t st) {
    dot_kernel<<<nblocks, kReduceThreads, 0, st>>>(n, x, y, partials);
    CCSD_LAUNCH_CHECK();
}

void k_sum(int n, const double *partials, double *out, cudaStream_t st) {
    sum_kernel<<<1, 1024, 0, st>>>(n, partials, out);
    CCSD_LAUNCH_CHECK();
}

void k_fill(size_t n, double val, double *p, cudaStream_t st) {
    if (n == 0) return;
    fill_kernel<<<grid_for(n), 256, 0, st>>>(n, val, p);
    CCSD_LAUNCH_CHECK();
}

void k_copy_diag(int n, const double *fock, int off, int cnt, double *out, cudaStream_t st) {
    copy_diag_kernel<<<(cnt + 255) / 256, 256, 0, st>>>(n, fock, off, cnt, out);
    CCSD_LAUNCH_CHECK();
}

}  // namespace ccsd
