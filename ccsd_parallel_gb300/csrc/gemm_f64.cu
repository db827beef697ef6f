// FP64 contraction kernel of the plain-FP64 path.
//
// C(m,n) = alpha * sum_k A(m,k) B(n,k) + beta * C(m,n), with A, B and C read
// and written through 3-level index views (common.h), so a 4-index CCSD
// contraction runs without a transposed copy.  tcgen05 has no f64 kind, so
// this path runs a 64x64 block tile with a 16-deep K step either as DFMA on the
// CUDA cores (4x4 register micro-tile per thread) or as mma.sync m8n8k4 DMMA on
// the FP64 tensor pipe (ccsd_set_fp64_kernel).  Skinny shapes are split over K
// into a scratch buffer and summed in a fixed order (deterministic results).
#include <atomic>

#include "../../include/ccsd_gb300.h"
#include "common.h"

namespace ccsd {

// the tiled kernel's inner product: CCSD_FP64_DFMA (CUDA cores) or CCSD_FP64_DMMA
// (mma.sync m8n8k4 on the FP64 tensor pipe); process-wide, ccsd_set_fp64_kernel
std::atomic<int> g_fp64_kernel{CCSD_FP64_DFMA};

namespace {

constexpr int BM = 64, BN = 64, BK = 16, NT = 256;

template <bool A_KC, bool B_KC>
__global__ void __launch_bounds__(NT) gemm_f64_kernel(int M, int N, int K, int kchunk,
                                                        double alpha, MatView A, MatView B,
                                                        double beta, OutView C, double *ws) {
    __shared__ double As[BK][BM + 1];
    __shared__ double Bs[BK][BN + 1];
    const int tid = threadIdx.x;
    const int tx = tid % 16, ty = tid / 16;
    const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
    const int kbeg = blockIdx.z * kchunk;
    const int kend = min(K, kbeg + kchunk);

    // Load mapping. K-contiguous operand: thread reads k = tid%16 of rows
    // tid/16 + 16q; otherwise m = tid%64 of k = tid/64 + 4q.
    int64_t a_row[4], b_row[4];
    bool a_ok[4], b_ok[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        int ra = A_KC ? (tid / 16 + 16 * q) : (tid % 64);
        int rb = B_KC ? (tid / 16 + 16 * q) : (tid % 64);
        a_ok[q] = (m0 + ra) < M;
        b_ok[q] = (n0 + rb) < N;
        a_row[q] = a_ok[q] ? dim_off(A.row, m0 + ra) : 0;
        b_row[q] = b_ok[q] ? dim_off(B.row, n0 + rb) : 0;
    }

    double acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;

    for (int k0 = kbeg; k0 < kend; k0 += BK) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            int ka = A_KC ? (tid % 16) : (tid / 64 + 4 * q);
            int ra = A_KC ? (tid / 16 + 16 * q) : (tid % 64);
            int kk = k0 + ka;
            double va = 0.0;
            if (a_ok[q] && kk < kend) va = A.p[a_row[q] + dim_off(A.col, kk)];
            As[ka][ra] = va;
            int kb = B_KC ? (tid % 16) : (tid / 64 + 4 * q);
            int rb = B_KC ? (tid / 16 + 16 * q) : (tid % 64);
            int kk2 = k0 + kb;
            double vb = 0.0;
            if (b_ok[q] && kk2 < kend) vb = B.p[b_row[q] + dim_off(B.col, kk2)];
            Bs[kb][rb] = vb;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; ++kk) {
            double a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }

    if (gridDim.z == 1) {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            int m = m0 + ty + 16 * i;
            if (m >= M) continue;
            int64_t ro = dim_off(C.row, m);
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                int n = n0 + tx + 16 * j;
                if (n >= N) continue;
                double *c = C.p + ro + dim_off(C.col, n);
                double v = alpha * acc[i][j];
                if (beta != 0.0) v = fma(beta, *c, v);
                *c = v;
            }
        }
    } else {
        double *w = ws + (size_t)blockIdx.z * M * N;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            int m = m0 + ty + 16 * i;
            if (m >= M) continue;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                int n = n0 + tx + 16 * j;
                if (n < N) w[(size_t)m * N + n] = acc[i][j];
            }
        }
    }
}

// The same tile on the FP64 tensor pipe: mma.sync m8n8k4 (DMMA).  The staging into
// shared memory is the DFMA kernel's; each of the 8 warps owns a 32 x 16 block of the
// 64 x 64 tile (4 x 2 fragments of 8 x 8, two accumulators per thread and fragment).
// Fragment layouts (PTX ISA, mma.m8n8k4 .f64): A row-major, lane holds A[lane/4][lane%4];
// B column-major, lane holds B[k = lane%4][n = lane/4]; C lane holds C[lane/4][2 (lane%4) + e].
template <bool A_KC, bool B_KC>
__global__ void __launch_bounds__(NT) gemm_f64_dmma_kernel(int M, int N, int K, int kchunk, double alpha,
                                                           MatView A, MatView B, double beta, OutView C,
                                                           double *ws) {
    __shared__ double As[BK][BM + 1];
    __shared__ double Bs[BK][BN + 1];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int wm = (warp & 1) * 32, wn = (warp >> 1) * 16;
    const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
    const int kbeg = blockIdx.z * kchunk;
    const int kend = min(K, kbeg + kchunk);

    int64_t a_row[4], b_row[4];
    bool a_ok[4], b_ok[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        int ra = A_KC ? (tid / 16 + 16 * q) : (tid % 64);
        int rb = B_KC ? (tid / 16 + 16 * q) : (tid % 64);
        a_ok[q] = (m0 + ra) < M;
        b_ok[q] = (n0 + rb) < N;
        a_row[q] = a_ok[q] ? dim_off(A.row, m0 + ra) : 0;
        b_row[q] = b_ok[q] ? dim_off(B.row, n0 + rb) : 0;
    }

    double acc[4][2][2];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) acc[i][j][0] = acc[i][j][1] = 0.0;

    const int fr = lane >> 2, fk = lane & 3;
    for (int k0 = kbeg; k0 < kend; k0 += BK) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            int ka = A_KC ? (tid % 16) : (tid / 64 + 4 * q);
            int ra = A_KC ? (tid / 16 + 16 * q) : (tid % 64);
            int kk = k0 + ka;
            double va = 0.0;
            if (a_ok[q] && kk < kend) va = A.p[a_row[q] + dim_off(A.col, kk)];
            As[ka][ra] = va;
            int kb = B_KC ? (tid % 16) : (tid / 64 + 4 * q);
            int rb = B_KC ? (tid / 16 + 16 * q) : (tid % 64);
            int kk2 = k0 + kb;
            double vb = 0.0;
            if (b_ok[q] && kk2 < kend) vb = B.p[b_row[q] + dim_off(B.col, kk2)];
            Bs[kb][rb] = vb;
        }
        __syncthreads();
#pragma unroll
        for (int ks = 0; ks < BK; ks += 4) {
            double a[4], b[2];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = As[ks + fk][wm + 8 * i + fr];
#pragma unroll
            for (int j = 0; j < 2; ++j) b[j] = Bs[ks + fk][wn + 8 * j + fr];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 2; ++j)
                    asm volatile(
                        "mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};\n"
                        : "+d"(acc[i][j][0]), "+d"(acc[i][j][1])
                        : "d"(a[i]), "d"(b[j]));
        }
        __syncthreads();
    }

#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int m = m0 + wm + 8 * i + fr;
        if (m >= M) continue;
        const int64_t ro = gridDim.z == 1 ? dim_off(C.row, m) : 0;
#pragma unroll
        for (int j = 0; j < 2; ++j) {
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                const int n = n0 + wn + 8 * j + 2 * fk + e;
                if (n >= N) continue;
                if (gridDim.z == 1) {
                    double *c = C.p + ro + dim_off(C.col, n);
                    double v = alpha * acc[i][j][e];
                    if (beta != 0.0) v = fma(beta, *c, v);
                    *c = v;
                } else {
                    ws[(size_t)blockIdx.z * M * N + (size_t)m * N + n] = acc[i][j][e];
                }
            }
        }
    }
}

__global__ void splitk_reduce_kernel(int M, int N, int splits, double alpha, const double *ws,
                                     double beta, OutView C) {
    size_t total = (size_t)M * N;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
         idx += (size_t)gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int z = 0; z < splits; ++z) s += ws[z * total + idx];
        int m = (int)(idx / N), n = (int)(idx % N);
        double *c = C.p + dim_off(C.row, m) + dim_off(C.col, n);
        double v = alpha * s;
        if (beta != 0.0) v = fma(beta, *c, v);
        *c = v;
    }
}

// Matrix-vector form (N == 1): y(m) = alpha sum_k A(m,k) x(k) + beta y(m).
// Memory-bound, so the reads follow the contiguous index of A:
//  ROWC: A(m,k) contiguous in m -> a block covers 32 rows x 8 k-slices, every
//        warp load is 32 consecutive rows, the 8 slices meet in shared memory;
//  else: one warp per row, lanes stride over k.
template <bool ROWC>
__global__ void __launch_bounds__(256) gemv_f64_kernel(int M, int K, double alpha, MatView A, MatView X,
                                                       double beta, OutView Y) {
    if (ROWC) {
        __shared__ double part[8][33];
        const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
        const int m = blockIdx.x * 32 + tx;
        double acc = 0.0;
        if (m < M) {
            // four independent chains keep four loads per thread in flight
            const int64_t ro = dim_off(A.row, m);
            double a1 = 0.0, a2 = 0.0, a3 = 0.0;
            int k = ty;
            for (; k + 24 < K; k += 32) {
                acc = fma(A.p[ro + dim_off(A.col, k)], X.p[dim_off(X.col, k)], acc);
                a1 = fma(A.p[ro + dim_off(A.col, k + 8)], X.p[dim_off(X.col, k + 8)], a1);
                a2 = fma(A.p[ro + dim_off(A.col, k + 16)], X.p[dim_off(X.col, k + 16)], a2);
                a3 = fma(A.p[ro + dim_off(A.col, k + 24)], X.p[dim_off(X.col, k + 24)], a3);
            }
            for (; k < K; k += 8) acc = fma(A.p[ro + dim_off(A.col, k)], X.p[dim_off(X.col, k)], acc);
            acc = (acc + a1) + (a2 + a3);
        }
        part[ty][tx] = acc;
        __syncthreads();
        if (ty == 0 && m < M) {
            double s = 0.0;
#pragma unroll
            for (int q = 0; q < 8; ++q) s += part[q][tx];
            double *y = Y.p + dim_off(Y.row, m) + dim_off(Y.col, 0);
            double v = alpha * s;
            if (beta != 0.0) v = fma(beta, *y, v);
            *y = v;
        }
    } else {
        const int lane = threadIdx.x & 31;
        const int m = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
        if (m >= M) return;
        const int64_t ro = dim_off(A.row, m);
        double acc = 0.0;
        for (int k = lane; k < K; k += 32) acc = fma(A.p[ro + dim_off(A.col, k)], X.p[dim_off(X.col, k)], acc);
        for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
        if (lane == 0) {
            double *y = Y.p + dim_off(Y.row, m) + dim_off(Y.col, 0);
            double v = alpha * acc;
            if (beta != 0.0) v = fma(beta, *y, v);
            *y = v;
        }
    }
}

// ROWC matrix-vector form with K split: a block covers 1024 consecutive rows (each
// thread 4 rows, 256 apart), so every k reads 8 KB of A contiguously; grid.y splits
// K so that the grid holds several blocks per SM.  With grid.y > 1 each block
// writes its partial sums to ws[y][m], added by splitk_reduce_kernel in a fixed
// order.
constexpr int GV_RW = 1024;
__global__ void __launch_bounds__(256) gemv_rowc_split_kernel(int M, int K, int kchunk, double alpha, MatView A,
                                                              MatView X, double beta, OutView Y, double *ws) {
    const int m0 = blockIdx.x * GV_RW + threadIdx.x;
    const int kbeg = blockIdx.y * kchunk, kend = min(K, kbeg + kchunk);
    int64_t ro[4];
    bool ok[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        ok[q] = m0 + 256 * q < M;
        ro[q] = ok[q] ? dim_off(A.row, m0 + 256 * q) : 0;
    }
    double acc[4] = {0.0, 0.0, 0.0, 0.0}, acc2[4] = {0.0, 0.0, 0.0, 0.0};
    int k = kbeg;
    for (; k + 1 < kend; k += 2) {
        const int64_t c0 = dim_off(A.col, k), c1 = dim_off(A.col, k + 1);
        const double x0 = X.p[dim_off(X.col, k)], x1 = X.p[dim_off(X.col, k + 1)];
        double a0[4], a1[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            a0[q] = ok[q] ? A.p[ro[q] + c0] : 0.0;
            a1[q] = ok[q] ? A.p[ro[q] + c1] : 0.0;
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            acc[q] = fma(a0[q], x0, acc[q]);
            acc2[q] = fma(a1[q], x1, acc2[q]);
        }
    }
    if (k < kend) {
        const int64_t c0 = dim_off(A.col, k);
        const double x0 = X.p[dim_off(X.col, k)];
#pragma unroll
        for (int q = 0; q < 4; ++q)
            if (ok[q]) acc[q] = fma(A.p[ro[q] + c0], x0, acc[q]);
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        if (!ok[q]) continue;
        const int m = m0 + 256 * q;
        const double sum = acc[q] + acc2[q];
        if (gridDim.y == 1) {
            double *y = Y.p + dim_off(Y.row, m) + dim_off(Y.col, 0);
            double v = alpha * sum;
            if (beta != 0.0) v = fma(beta, *y, v);
            *y = v;
        } else {
            ws[(size_t)blockIdx.y * M + m] = sum;
        }
    }
}

// Skinny form (N <= 16 columns, long K): the contraction streams A once and is
// memory-bound.  A block covers 32 rows (4 per warp) and one K range; for each
// 128-wide k chunk it stages B(0..N-1, k) in shared memory, and every lane
// accumulates 4 rows x NN columns over k = lane + 32 q, so consecutive lanes read
// consecutive k of A (coalesced when A is K-contiguous) and one column offset
// serves four rows.  Lanes meet in a warp reduction at the end; a K-split writes
// per-range partial sums that splitk_reduce_kernel adds in a fixed order.
constexpr int SK_ROWS = 4, SK_KC = 128;

template <int NN>
__global__ void __launch_bounds__(256) gemm_skinny_f64_kernel(int M, int N, int K, int kchunk, double alpha,
                                                              MatView A, MatView B, double beta, OutView C,
                                                              double *ws) {
    __shared__ double Bs[NN][SK_KC];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int m0 = blockIdx.x * (8 * SK_ROWS) + warp * SK_ROWS;
    const int kbeg = blockIdx.y * kchunk;
    const int kend = min(K, kbeg + kchunk);
    int64_t arow[SK_ROWS];
    bool aok[SK_ROWS];
#pragma unroll
    for (int r = 0; r < SK_ROWS; ++r) {
        aok[r] = m0 + r < M;
        arow[r] = aok[r] ? dim_off(A.row, m0 + r) : 0;
    }
    double acc[SK_ROWS][NN];
#pragma unroll
    for (int r = 0; r < SK_ROWS; ++r)
#pragma unroll
        for (int n = 0; n < NN; ++n) acc[r][n] = 0.0;

    for (int k0 = kbeg; k0 < kend; k0 += SK_KC) {
        __syncthreads();
        for (int e = threadIdx.x; e < NN * SK_KC; e += blockDim.x) {
            const int n = e / SK_KC, kk = e % SK_KC, k = k0 + kk;
            Bs[n][kk] = (n < N && k < kend) ? B.p[dim_off(B.row, n) + dim_off(B.col, k)] : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int q = 0; q < SK_KC / 32; ++q) {
            const int kk = lane + 32 * q, k = k0 + kk;
            if (k < kend) {
                const int64_t co = dim_off(A.col, k);
                double a[SK_ROWS];
#pragma unroll
                for (int r = 0; r < SK_ROWS; ++r) a[r] = aok[r] ? A.p[arow[r] + co] : 0.0;
#pragma unroll
                for (int n = 0; n < NN; ++n) {
                    const double b = Bs[n][kk];
#pragma unroll
                    for (int r = 0; r < SK_ROWS; ++r) acc[r][n] = fma(a[r], b, acc[r][n]);
                }
            }
        }
    }
#pragma unroll
    for (int r = 0; r < SK_ROWS; ++r)
#pragma unroll
        for (int n = 0; n < NN; ++n)
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) acc[r][n] += __shfl_down_sync(0xffffffffu, acc[r][n], off);
    if (lane != 0) return;
#pragma unroll
    for (int r = 0; r < SK_ROWS; ++r) {
        const int m = m0 + r;
        if (m >= M) continue;
        if (gridDim.y == 1) {
            const int64_t ro = dim_off(C.row, m);
#pragma unroll
            for (int n = 0; n < NN; ++n) {
                if (n >= N) break;
                double *c = C.p + ro + dim_off(C.col, n);
                double v = alpha * acc[r][n];
                if (beta != 0.0) v = fma(beta, *c, v);
                *c = v;
            }
        } else {
            double *w = ws + (size_t)blockIdx.y * M * N + (size_t)m * N;
#pragma unroll
            for (int n = 0; n < NN; ++n)
                if (n < N) w[n] = acc[r][n];
        }
    }
}

// Thin form (N <= 16 columns, K <= 64, many rows): the product streams A and C
// once, with about 2 N flops per byte.  One thread per row of A; the N x K block
// of B and the column offsets of A and C sit in shared memory, so a warp reads 32
// rows at each k and writes its rows' N outputs with no reduction.
constexpr int TH_KMAX = 64;

template <int NN>
__global__ void __launch_bounds__(256) gemm_thin_f64_kernel(int M, int N, int K, double alpha, MatView A,
                                                            MatView B, double beta, OutView C) {
    __shared__ double bs[TH_KMAX][NN];
    __shared__ int64_t ak[TH_KMAX];
    __shared__ int64_t cn[NN];
    for (int e = threadIdx.x; e < K * NN; e += blockDim.x) {
        const int k = e / NN, n = e % NN;
        bs[k][n] = n < N ? B.p[dim_off(B.row, n) + dim_off(B.col, k)] : 0.0;
    }
    for (int k = threadIdx.x; k < K; k += blockDim.x) ak[k] = dim_off(A.col, k);
    for (int n = threadIdx.x; n < NN; n += blockDim.x) cn[n] = n < N ? dim_off(C.col, n) : 0;
    __syncthreads();
    for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < M; m += gridDim.x * blockDim.x) {
        const double *a = A.p + dim_off(A.row, m);
        double acc[NN];
#pragma unroll
        for (int n = 0; n < NN; ++n) acc[n] = 0.0;
        for (int k = 0; k < K; ++k) {
            const double x = a[ak[k]];
#pragma unroll
            for (int n = 0; n < NN; ++n) acc[n] = fma(x, bs[k][n], acc[n]);
        }
        double *c = C.p + dim_off(C.row, m);
#pragma unroll
        for (int n = 0; n < NN; ++n) {
            if (n >= N) break;
            double v = alpha * acc[n];
            if (beta != 0.0) v = fma(beta, c[cn[n]], v);
            c[cn[n]] = v;
        }
    }
}

bool thin_shape(int M, int N, int K) {
    const int lo = M < N ? M : N, hi = M < N ? N : M;
    return lo <= 16 && hi >= 256 && K <= TH_KMAX;
}

template <int NN>
void launch_thin(int M, int N, int K, double alpha, const MatView &A, const MatView &B, double beta,
                 const OutView &C, cudaStream_t st) {
    const int blocks = (int)std::min<long>((M + 255) / 256, 152L * 8);
    gemm_thin_f64_kernel<NN><<<blocks, 256, 0, st>>>(M, N, K, alpha, A, B, beta, C);
    CCSD_LAUNCH_CHECK();
}

constexpr int kTargetBlocks = 2 * 152;
constexpr int kSkinnyMaxN = 16;

// K ranges for the skinny form: enough blocks to cover the SMs four times over.
int choose_skinny_splits(int M, int K) {
    const long mblocks = (M + 8 * SK_ROWS - 1) / (8 * SK_ROWS);
    const long want = (4 * 152 + mblocks - 1) / mblocks;
    const long maxk = (K + 4 * SK_KC - 1) / (4 * SK_KC);  // at least four chunks per range
    long s = want < maxk ? want : maxk;
    if (s > 128) s = 128;
    return s < 1 ? 1 : (int)s;
}

// The skinny form takes a shape whose short side is at most 16 and whose other
// sides are long enough for it to matter (the tiled kernel wastes most of a 64-wide
// tile there); returns the number of columns after orienting the short side to N.
bool skinny_shape(int M, int N, int K) {
    const int lo = M < N ? M : N, hi = M < N ? N : M;
    return lo <= kSkinnyMaxN && hi >= 64 && K >= 256;
}

// K ranges for the tiled kernel: enough blocks for two per SM.  One SM's FP64 pipe
// does about 8 GFLOP/s, so a 64 x 64 tile over K = 300 alone takes 80 us; ranges go
// down to one 16-deep K step when there are few tiles.
int choose_splits(int M, int N, int K) {
    long tiles = (long)((M + BM - 1) / BM) * ((N + BN - 1) / BN);
    if (tiles >= kTargetBlocks) return 1;
    long want = (kTargetBlocks + tiles - 1) / tiles;
    long maxk = (K + BK - 1) / BK;
    long s = want < maxk ? want : maxk;
    if (s > 64) s = 64;
    return s < 1 ? 1 : (int)s;
}

}  // namespace

size_t gemm_f64_ws_elems(int M, int N, int K) {
    if (M > 1 && N > 1 && thin_shape(M, N, K)) return 0;
    if (skinny_shape(M, N, K)) {
        const int Ml = M < N ? N : M;
        int s = choose_skinny_splits(Ml, K);
        return s > 1 ? (size_t)s * M * N : 0;
    }
    if (M == 1 || N == 1) return (size_t)std::max(M, N) * 64;  // the K-split matrix-vector form
    int s = choose_splits(M, N, K);
    return s > 1 ? (size_t)s * M * N : 0;
}

namespace {
template <int NN>
void launch_skinny(int M, int N, int K, double alpha, const MatView &A, const MatView &B, double beta,
                   const OutView &C, double *ws, size_t ws_elems, cudaStream_t st) {
    int splits = choose_skinny_splits(M, K);
    while (splits > 1 && (size_t)splits * M * N > ws_elems) --splits;
    int kchunk = (K + splits - 1) / splits;
    kchunk = (kchunk + SK_KC - 1) / SK_KC * SK_KC;
    splits = (K + kchunk - 1) / kchunk;
    dim3 grid((M + 8 * SK_ROWS - 1) / (8 * SK_ROWS), splits);
    gemm_skinny_f64_kernel<NN><<<grid, 256, 0, st>>>(M, N, K, kchunk, alpha, A, B, beta, C, ws);
    CCSD_LAUNCH_CHECK();
    if (splits > 1) {
        size_t total = (size_t)M * N;
        int blocks = (int)std::min<size_t>((total + 255) / 256, 4096);
        splitk_reduce_kernel<<<blocks, 256, 0, st>>>(M, N, splits, alpha, ws, beta, C);
        CCSD_LAUNCH_CHECK();
    }
}
}  // namespace

void gemm_f64(int M, int N, int K, double alpha, const MatView &A, const MatView &B, double beta,
              const OutView &C, double *ws, size_t ws_elems, cudaStream_t st) {
    if (M <= 0 || N <= 0) return;
    if (K <= 0) {
        axpby_view(M, N, 0.0, MatView{C.p, C.row, C.col}, beta, C, st);
        return;
    }
    if (N == 1 || M == 1) {
        // matrix-vector: put the long side in the rows of the view
        const MatView &Am = N == 1 ? A : B;
        const MatView &Xv = N == 1 ? B : A;
        const OutView Y = N == 1 ? C : OutView{C.p, C.col, C.row};
        const int R = N == 1 ? M : N;
        if (Am.row.s2 == 1 && Am.col.s2 != 1) {
            // K split until the grid holds about 8 blocks per SM, the loads in flight that
            // HBM latency needs (deterministic partials in ws)
            const int gx = (R + GV_RW - 1) / GV_RW;
            int splits = std::max(1, std::min((8 * 152 + gx - 1) / gx, K / 64));
            while (splits > 1 && (size_t)splits * R > ws_elems) --splits;
            const int kchunk = (K + splits - 1) / splits;
            splits = (K + kchunk - 1) / kchunk;
            gemv_rowc_split_kernel<<<dim3(gx, splits), 256, 0, st>>>(R, K, kchunk, alpha, Am, Xv, beta, Y, ws);
            CCSD_LAUNCH_CHECK();
            if (splits > 1) {
                splitk_reduce_kernel<<<(R + 255) / 256, 256, 0, st>>>(R, 1, splits, alpha, ws, beta, Y);
                CCSD_LAUNCH_CHECK();
            }
            return;
        } else if (skinny_shape(R, 1, K) && R < 8 * 152 * 8) {
            // few rows of a long K: the K-split skinny form keeps every SM busy
            launch_skinny<1>(R, 1, K, alpha, Am, Xv, beta, Y, ws, ws_elems, st);
            return;
        } else {
            gemv_f64_kernel<false><<<(R + 7) / 8, 256, 0, st>>>(R, K, alpha, Am, Xv, beta, Y);
        }
        CCSD_LAUNCH_CHECK();
        return;
    }
    if (thin_shape(M, N, K)) {
        if (M < N) {  // the short side goes to the columns
            gemm_f64(N, M, K, alpha, B, A, beta, OutView{C.p, C.col, C.row}, ws, ws_elems, st);
            return;
        }
        if (N <= 2) launch_thin<2>(M, N, K, alpha, A, B, beta, C, st);
        else if (N <= 4) launch_thin<4>(M, N, K, alpha, A, B, beta, C, st);
        else if (N <= 8) launch_thin<8>(M, N, K, alpha, A, B, beta, C, st);
        else launch_thin<16>(M, N, K, alpha, A, B, beta, C, st);
        return;
    }
    if (skinny_shape(M, N, K)) {
        if (M < N) {  // the short side goes to the columns
            gemm_f64(N, M, K, alpha, B, A, beta, OutView{C.p, C.col, C.row}, ws, ws_elems, st);
            return;
        }
        if (N <= 2) launch_skinny<2>(M, N, K, alpha, A, B, beta, C, ws, ws_elems, st);
        else if (N <= 4) launch_skinny<4>(M, N, K, alpha, A, B, beta, C, ws, ws_elems, st);
        else if (N <= 8) launch_skinny<8>(M, N, K, alpha, A, B, beta, C, ws, ws_elems, st);
        else launch_skinny<16>(M, N, K, alpha, A, B, beta, C, ws, ws_elems, st);
        return;
    }
    if ((N + BN - 1) / BN > 65535) {  // grid.y limit: the long side goes to grid.x
        if ((M + BN - 1) / BN > 65535) throw Error(CCSD_ERR_INVALID_ARG, "FP64 GEMM beyond the launch grid");
        gemm_f64(N, M, K, alpha, B, A, beta, OutView{C.p, C.col, C.row}, ws, ws_elems, st);
        return;
    }
    int splits = choose_splits(M, N, K);
    while (splits > 1 && (size_t)splits * M * N > ws_elems) --splits;
    int kchunk = (K + splits - 1) / splits;
    kchunk = (kchunk + BK - 1) / BK * BK;
    splits = (K + kchunk - 1) / kchunk;
    dim3 grid((M + BM - 1) / BM, (N + BN - 1) / BN, splits);
    bool akc = A.col.s2 == 1;
    bool bkc = B.col.s2 == 1;
    if (g_fp64_kernel.load(std::memory_order_relaxed) == CCSD_FP64_DMMA) {
        if (akc && bkc)
            gemm_f64_dmma_kernel<true, true><<<grid, NT, 0, st>>>(M, N, K, kchunk, alpha, A, B, beta, C, ws);
        else if (akc)
            gemm_f64_dmma_kernel<true, false><<<grid, NT, 0, st>>>(M, N, K, kchunk, alpha, A, B, beta, C, ws);
        else if (bkc)
            gemm_f64_dmma_kernel<false, true><<<grid, NT, 0, st>>>(M, N, K, kchunk, alpha, A, B, beta, C, ws);
        else
            gemm_f64_dmma_kernel<false, false><<<grid, NT, 0, st>>>(M, N, K, kchunk, alpha, A, B, beta, C, ws);
    } else if (akc && bkc)
        gemm_f64_kernel<true, true><<<grid, NT, 0, st>>>(M, N, K, kchunk, alpha, A, B, beta, C, ws);
    else if (akc)
        gemm_f64_kernel<true, false><<<grid, NT, 0, st>>>(M, N, K, kchunk, alpha, A, B, beta, C, ws);
    else if (bkc)
        gemm_f64_kernel<false, true><<<grid, NT, 0, st>>>(M, N, K, kchunk, alpha, A, B, beta, C, ws);
    else
        gemm_f64_kernel<false, false><<<grid, NT, 0, st>>>(M, N, K, kchunk, alpha, A, B, beta, C, ws);
    CCSD_LAUNCH_CHECK();
    if (splits > 1) {
        size_t total = (size_t)M * N;
        int blocks = (int)std::min<size_t>((total + 255) / 256, 4096);
        splitk_reduce_kernel<<<blocks, 256, 0, st>>>(M, N, splits, alpha, ws, beta, C);
        CCSD_LAUNCH_CHECK();
    }
}

}  // namespace ccsd

extern "C" int ccsd_set_fp64_kernel(int32_t kind) {
    if (kind != CCSD_FP64_DFMA && kind != CCSD_FP64_DMMA) return CCSD_ERR_INVALID_ARG;
    return ccsd::g_fp64_kernel.exchange(kind);
}
