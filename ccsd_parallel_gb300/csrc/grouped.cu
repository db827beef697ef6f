// Grouped kernels of the batched solve (grouped.h).
//
// The contraction kernel is persistent: a grid of (SMs x resident blocks)
// walks one flat list of work items, each a (system, tile row, tile column,
// K slice) of that system's contraction, so systems of uneven nocc/nvir share
// one launch without idle tails.  Split-K partials go to a scratch buffer and
// are summed in a fixed order (results do not depend on scheduling).  The
// element-wise kernels put the system in blockIdx.y.
#include <algorithm>

#include "grouped.h"
#include "ladder_sym.cuh"

namespace ccsd {

namespace {

constexpr int kThreads = 256;
constexpr int kBK = 16;
constexpr int kUpdBlocks = 32;               // t2 partial sums per system
constexpr int kPer = kUpdBlocks + 1;         // + the t1 partial

__device__ __forceinline__ int find_part(const GGemm *parts, int nparts, int item) {
    int lo = 0, hi = nparts - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (parts[mid].item_begin <= item) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

template <int TM, int TN, bool A_KC, bool B_KC>
__global__ void __launch_bounds__(kThreads) ggemm_kernel(const GGemm *__restrict__ parts, int nparts, int total,
                                                          const int *__restrict__ active, double *__restrict__ ws) {
    constexpr int BM = 16 * TM, BN = 16 * TN;
    __shared__ double As[kBK][BM + 1];
    __shared__ double Bs[kBK][BN + 1];
    __shared__ int s_part;
    const int tid = threadIdx.x;
    const int tx = tid % 16, ty = tid / 16;
    for (int item = blockIdx.x; item < total; item += gridDim.x) {
        if (tid == 0) s_part = find_part(parts, nparts, item);
        __syncthreads();
        const GGemm &g = parts[s_part];
        const bool run = active[g.sys] != 0;
        if (run) {
            const int M = g.M, N = g.N, K = g.K;
            const int local = item - g.item_begin;
            const int per = g.tiles_m * g.tiles_n;
            const int z = local / per, r = local % per;
            const int m0 = (r / g.tiles_n) * BM, n0 = (r % g.tiles_n) * BN;
            const int kbeg = z * g.kchunk;
            const int kend = min(K, kbeg + g.kchunk);
            const MatView A = g.A, B = g.B;

            int64_t a_row[TM], b_row[TN];
            bool a_ok[TM], b_ok[TN];
#pragma unroll
            for (int q = 0; q < TM; ++q) {
                const int e = tid + kThreads * q;
                const int ra = A_KC ? e / kBK : e % BM;
                a_ok[q] = (m0 + ra) < M;
                a_row[q] = a_ok[q] ? dim_off(A.row, m0 + ra) : 0;
            }
#pragma unroll
            for (int q = 0; q < TN; ++q) {
                const int e = tid + kThreads * q;
                const int rb = B_KC ? e / kBK : e % BN;
                b_ok[q] = (n0 + rb) < N;
                b_row[q] = b_ok[q] ? dim_off(B.row, n0 + rb) : 0;
            }
            double acc[TM][TN];
#pragma unroll
            for (int i = 0; i < TM; ++i)
#pragma unroll
                for (int j = 0; j < TN; ++j) acc[i][j] = 0.0;

            for (int k0 = kbeg; k0 < kend; k0 += kBK) {
#pragma unroll
                for (int q = 0; q < TM; ++q) {
                    const int e = tid + kThreads * q;
                    const int ra = A_KC ? e / kBK : e % BM;
                    const int ka = A_KC ? e % kBK : e / BM;
                    const int kk = k0 + ka;
                    As[ka][ra] = (a_ok[q] && kk < kend) ? A.p[a_row[q] + dim_off(A.col, kk)] : 0.0;
                }
#pragma unroll
                for (int q = 0; q < TN; ++q) {
                    const int e = tid + kThreads * q;
                    const int rb = B_KC ? e / kBK : e % BN;
                    const int kb = B_KC ? e % kBK : e / BN;
                    const int kk = k0 + kb;
                    Bs[kb][rb] = (b_ok[q] && kk < kend) ? B.p[b_row[q] + dim_off(B.col, kk)] : 0.0;
                }
                __syncthreads();
#pragma unroll
                for (int kk = 0; kk < kBK; ++kk) {
                    double a[TM], b[TN];
#pragma unroll
                    for (int i = 0; i < TM; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
                    for (int j = 0; j < TN; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
                    for (int i = 0; i < TM; ++i)
#pragma unroll
                        for (int j = 0; j < TN; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
                }
                __syncthreads();
            }

            if (g.splits == 1) {
                const double alpha = g.alpha, beta = g.beta;
#pragma unroll
                for (int i = 0; i < TM; ++i) {
                    const int m = m0 + ty + 16 * i;
                    if (m >= M) continue;
                    const int64_t ro = dim_off(g.C.row, m);
#pragma unroll
                    for (int j = 0; j < TN; ++j) {
                        const int n = n0 + tx + 16 * j;
                        if (n >= N) continue;
                        double *c = g.C.p + ro + dim_off(g.C.col, n);
                        double v = alpha * acc[i][j];
                        if (beta != 0.0) v = fma(beta, *c, v);
                        *c = v;
                    }
                }
            } else {
                double *w = ws + g.ws_off + (size_t)z * M * N;
#pragma unroll
                for (int i = 0; i < TM; ++i) {
                    const int m = m0 + ty + 16 * i;
                    if (m >= M) continue;
#pragma unroll
                    for (int j = 0; j < TN; ++j) {
                        const int n = n0 + tx + 16 * j;
                        if (n < N) w[(size_t)m * N + n] = acc[i][j];
                    }
                }
            }
        }
        __syncthreads();  // s_part is rewritten by the next item
    }
}

__global__ void ggemm_reduce_kernel(const GGemm *__restrict__ parts, const int *__restrict__ active,
                                    const double *__restrict__ ws) {
    const GGemm &g = parts[blockIdx.y];
    if (g.splits <= 1 || !active[g.sys]) return;
    const size_t total = (size_t)g.M * g.N;
    const double *w = ws + g.ws_off;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
         idx += (size_t)gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int z = 0; z < g.splits; ++z) s += w[z * total + idx];
        const int m = (int)(idx / g.N), n = (int)(idx % g.N);
        double *c = g.C.p + dim_off(g.C.row, m) + dim_off(g.C.col, n);
        double v = g.alpha * s;
        if (g.beta != 0.0) v = fma(g.beta, *c, v);
        *c = v;
    }
}

// Matrix-vector parts (M == 1 or N == 1): one warp per output element.
__global__ void ggemv_kernel(const GGemm *__restrict__ parts, const int *__restrict__ active) {
    const GGemm &g = parts[blockIdx.y];
    if (!active[g.sys]) return;
    const bool colvec = g.N == 1;  // y(m) = A(m,:) . B(0,:)
    const int rows = colvec ? g.M : g.N;
    const MatView &Am = colvec ? g.A : g.B;
    const MatView &Xv = colvec ? g.B : g.A;
    const int lane = threadIdx.x & 31;
    const int warps = blockDim.x >> 5;
    for (int r = blockIdx.x * warps + (threadIdx.x >> 5); r < rows; r += gridDim.x * warps) {
        const int64_t ro = dim_off(Am.row, r);
        double acc = 0.0;
        for (int k = lane; k < g.K; k += 32) acc = fma(Am.p[ro + dim_off(Am.col, k)], Xv.p[dim_off(Xv.col, k)], acc);
        for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
        if (lane == 0) {
            double *y = colvec ? g.C.p + dim_off(g.C.row, r) : g.C.p + dim_off(g.C.col, r);
            double v = g.alpha * acc;
            if (g.beta != 0.0) v = fma(g.beta, *y, v);
            *y = v;
        }
    }
}

__global__ void gaxpby_kernel(const GAxpby *__restrict__ parts, const int *__restrict__ active) {
    const GAxpby &g = parts[blockIdx.y];
    if (!active[g.sys]) return;
    const size_t total = (size_t)g.R * g.C;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
         idx += (size_t)gridDim.x * blockDim.x) {
        const uint32_t r = (uint32_t)(idx / g.C), c = (uint32_t)(idx % g.C);
        double *y = g.Y.p + dim_off(g.Y.row, r) + dim_off(g.Y.col, c);
        double v = g.alpha == 0.0 ? 0.0 : g.alpha * g.X.p[dim_off(g.X.row, r) + dim_off(g.X.col, c)];
        if (g.beta != 0.0) v = fma(g.beta, *y, v);
        *y = v;
    }
}

__global__ void gtau_kernel(const GAmp *__restrict__ parts, const int *__restrict__ active) {
    const GAmp &g = parts[blockIdx.y];
    if (!active[g.sys]) return;
    const int o = g.o, v = g.v;
    const size_t total = (size_t)o * o * v * v;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
         idx += (size_t)gridDim.x * blockDim.x) {
        const int b = idx % v;
        size_t r = idx / v;
        const int a = r % v;
        r /= v;
        const int j = r % o;
        const int i = (int)(r / o);
        g.out1[idx] = g.t2[idx] + g.t1[i * v + a] * g.t1[j * v + b];
    }
}

// th1[i,a,l,d] = t2[i,l,a,d] - t2[i,l,d,a]/2 - t1[i,d] t1[l,a]; th2[i,a,l,d] = t2[i,l,d,a]/2 + t1[i,d] t1[l,a]
__global__ void gtheta_kernel(const GAmp *__restrict__ parts, const int *__restrict__ active) {
    const GAmp &g = parts[blockIdx.y];
    if (!active[g.sys]) return;
    const int o = g.o, v = g.v;
    const size_t total = (size_t)o * v * o * v, ov2 = (size_t)o * v * v, v2 = (size_t)v * v;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
         idx += (size_t)gridDim.x * blockDim.x) {
        const int d = idx % v;
        size_t r = idx / v;
        const int l = r % o;
        r /= o;
        const int a = r % v;
        const int i = (int)(r / v);
        const double tad = g.t2[i * ov2 + l * v2 + (size_t)a * v + d];
        const double tda = g.t2[i * ov2 + l * v2 + (size_t)d * v + a];
        const double tt = g.t1[i * v + d] * g.t1[l * v + a];
        g.out1[idx] = tad - 0.5 * tda - tt;
        g.out2[idx] = 0.5 * tda + tt;
    }
}

__global__ void gtau_sym_kernel(const GAmp *__restrict__ parts, const int *__restrict__ active) {
    const GAmp &g = parts[blockIdx.y];
    if (!active[g.sys]) return;
    const int64_t total = (int64_t)g.o * (g.o + 1) / 2 * ((int64_t)g.v * (g.v + 1) / 2);
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x)
        pair::tau_sym_elem(g.o, g.v, g.t1, g.out1, g.out2, idx);
}

__global__ void gunpack_kernel(const GAmp *__restrict__ parts, const int *__restrict__ active) {
    const GAmp &g = parts[blockIdx.y];
    if (!active[g.sys]) return;
    const int64_t total = (int64_t)g.o * g.o * g.v * g.v;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x)
        pair::unpack_elem(g.o, g.v, g.t1, g.t2, g.out1, idx);
}

__device__ double gblock_sum(double x) {
    __shared__ double sh[32];
    for (int off = 16; off > 0; off >>= 1) x += __shfl_down_sync(0xffffffffu, x, off);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) sh[w] = x;
    __syncthreads();
    double s = 0.0;
    if (w == 0) {
        const int nw = blockDim.x >> 5;
        s = lane < nw ? sh[lane] : 0.0;
        for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
    }
    __syncthreads();
    return s;  // valid in thread 0
}

// blockIdx.x < kUpdBlocks: T2 slices; blockIdx.x == kUpdBlocks: T1.
__global__ void gupdate_kernel(const GUpdate *__restrict__ parts, const int *__restrict__ active,
                               double *__restrict__ partials) {
    const GUpdate &g = parts[blockIdx.y];
    if (!active[g.sys]) return;
    const int o = g.o, v = g.v;
    double acc = 0.0;
    if (blockIdx.x < kUpdBlocks) {
        const size_t total = (size_t)o * o * v * v, v2 = (size_t)v * v, ov2 = (size_t)o * v2;
        for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
             idx += (size_t)kUpdBlocks * blockDim.x) {
            const int b = idx % v;
            size_t r = idx / v;
            const int a = r % v;
            r /= v;
            const int j = r % o;
            const int i = (int)(r / o);
            const double num = g.R[idx] + g.Rp[idx] + g.Rp[j * ov2 + i * v2 + (size_t)b * v + a];
            const double t = num / (g.eo[i] + g.eo[j] - g.ev[a] - g.ev[b]);
            const double d = t - g.t2_old[idx];
            acc = fma(d, d, acc);
            g.t2_new[idx] = t;
        }
    } else {
        for (int idx = threadIdx.x; idx < o * v; idx += blockDim.x) {
            const int i = idx / v, a = idx % v;
            const double t = g.R1[idx] / (g.eo[i] - g.ev[a]);
            const double d = t - g.t1_old[idx];
            acc = fma(d, d, acc);
            g.t1_new[idx] = t;
        }
    }
    const double s = gblock_sum(acc);
    if (threadIdx.x == 0) partials[(size_t)blockIdx.y * kPer + blockIdx.x] = s;
}

__global__ void gdot_kernel(const GDot *__restrict__ parts, const int *__restrict__ active,
                            double *__restrict__ partials) {
    const GDot &g = parts[blockIdx.y];
    if (!active[g.sys]) return;
    double acc = 0.0;
    if (blockIdx.x < kUpdBlocks)
        for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < g.n;
             idx += (long long)kUpdBlocks * blockDim.x)
            acc = fma(g.x[idx], g.y[idx], acc);
    const double s = gblock_sum(acc);
    if (threadIdx.x == 0) partials[(size_t)blockIdx.y * kPer + blockIdx.x] = s;
}

__global__ void gsum_kernel(const int *__restrict__ active, const double *__restrict__ partials,
                            double *__restrict__ out) {
    if (!active[blockIdx.x]) return;
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int q = 0; q < kPer; ++q) s += partials[(size_t)blockIdx.x * kPer + q];
        out[blockIdx.x] = s;
    }
}

inline int grid_x(size_t max_elems) {
    size_t b = (max_elems + kThreads - 1) / kThreads;
    if (b > 256) b = 256;
    return b < 1 ? 1 : (int)b;
}

template <int TM, int TN>
void launch_tile(const GGemmPlan &p, const GGemm *d, int nparts, const int *active, double *ws, cudaStream_t st) {
    if (p.akc && p.bkc)
        ggemm_kernel<TM, TN, true, true><<<p.grid, kThreads, 0, st>>>(d, nparts, p.total_items, active, ws);
    else if (p.akc)
        ggemm_kernel<TM, TN, true, false><<<p.grid, kThreads, 0, st>>>(d, nparts, p.total_items, active, ws);
    else if (p.bkc)
        ggemm_kernel<TM, TN, false, true><<<p.grid, kThreads, 0, st>>>(d, nparts, p.total_items, active, ws);
    else
        ggemm_kernel<TM, TN, false, false><<<p.grid, kThreads, 0, st>>>(d, nparts, p.total_items, active, ws);
    CCSD_LAUNCH_CHECK();
}

template <int TM, int TN>
int occupancy() {
    int b = 1;
    CCSD_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, ggemm_kernel<TM, TN, true, true>, kThreads, 0));
    return b < 1 ? 1 : b;
}

int tile_occupancy(int cfg) {
    static int cache[kNumGTiles] = {0};
    if (!cache[cfg]) {
        switch (cfg) {
            case kTile64x64: cache[cfg] = occupancy<4, 4>(); break;
            case kTile32x64: cache[cfg] = occupancy<2, 4>(); break;
            case kTile64x32: cache[cfg] = occupancy<4, 2>(); break;
            case kTile32x32: cache[cfg] = occupancy<2, 2>(); break;
            default: cache[cfg] = occupancy<8, 4>(); break;
        }
    }
    return cache[cfg];
}

}  // namespace

int gtile_bm(int cfg) {
    static const int bm[kNumGTiles] = {64, 32, 64, 32, 128};
    return bm[cfg];
}
int gtile_bn(int cfg) {
    static const int bn[kNumGTiles] = {64, 64, 32, 32, 64};
    return bn[cfg];
}

GGemmPlan plan_grouped_gemm(std::vector<GGemm> &parts, int cfg, int target, int num_sms) {
    GGemmPlan p;
    p.cfg = cfg;
    p.target = target;
    p.gemv = !parts.empty();
    for (const GGemm &g : parts)
        if (g.M != 1 && g.N != 1) p.gemv = false;
    p.akc = !parts.empty() && parts[0].A.col.s2 == 1;
    p.bkc = !parts.empty() && parts[0].B.col.s2 == 1;
    for (const GGemm &g : parts) {  // the kernel variant needs one contiguity pattern
        if ((g.A.col.s2 == 1) != p.akc) p.akc = false;
        if ((g.B.col.s2 == 1) != p.bkc) p.bkc = false;
    }
    if (p.gemv) {
        for (GGemm &g : parts) {
            g.splits = 1;
            g.kchunk = g.K;
            g.tiles_m = g.tiles_n = 1;
        }
        return p;
    }
    const int BM = gtile_bm(cfg), BN = gtile_bn(cfg);
    long tiles = 0;
    for (GGemm &g : parts) {
        g.tiles_m = (g.M + BM - 1) / BM;
        g.tiles_n = (g.N + BN - 1) / BN;
        tiles += (long)g.tiles_m * g.tiles_n;
    }
    int s = 1;
    if (target > 0 && tiles < target) s = (int)std::min<long>(64, (target + tiles - 1) / tiles);
    int items = 0;
    size_t ws = 0;
    for (GGemm &g : parts) {
        int sp = std::max(1, std::min(s, g.K / 64));
        int kchunk = (g.K + sp - 1) / sp;
        kchunk = (kchunk + kBK - 1) / kBK * kBK;
        sp = (g.K + kchunk - 1) / kchunk;
        g.splits = sp;
        g.kchunk = kchunk;
        g.item_begin = items;
        items += sp * g.tiles_m * g.tiles_n;
        g.ws_off = 0;
        if (sp > 1) {
            g.ws_off = (long long)ws;
            ws += (size_t)sp * g.M * g.N;
            p.any_split = true;
        }
    }
    p.total_items = items;
    p.ws_elems = ws;
    const int resident = num_sms * tile_occupancy(cfg);
    p.grid = std::max(1, std::min(items, resident));
    return p;
}

void launch_grouped_gemm(const GGemmPlan &p, const GGemm *d, int nparts, const int *active, double *ws,
                         cudaStream_t st) {
    if (nparts <= 0) return;
    if (p.gemv) {
        ggemv_kernel<<<dim3(64, nparts), kThreads, 0, st>>>(d, active);
        CCSD_LAUNCH_CHECK();
        return;
    }
    if (p.total_items <= 0) return;
    switch (p.cfg) {
        case kTile64x64: launch_tile<4, 4>(p, d, nparts, active, ws, st); break;
        case kTile32x64: launch_tile<2, 4>(p, d, nparts, active, ws, st); break;
        case kTile64x32: launch_tile<4, 2>(p, d, nparts, active, ws, st); break;
        case kTile32x32: launch_tile<2, 2>(p, d, nparts, active, ws, st); break;
        default: launch_tile<8, 4>(p, d, nparts, active, ws, st); break;
    }
    if (p.any_split) {
        ggemm_reduce_kernel<<<dim3(32, nparts), kThreads, 0, st>>>(d, active, ws);
        CCSD_LAUNCH_CHECK();
    }
}

void launch_grouped_axpby(const GAxpby *d, int nparts, size_t max_elems, const int *active, cudaStream_t st) {
    if (nparts <= 0) return;
    gaxpby_kernel<<<dim3(grid_x(max_elems), nparts), kThreads, 0, st>>>(d, active);
    CCSD_LAUNCH_CHECK();
}

void launch_grouped_tau(const GAmp *d, int nparts, size_t max_elems, const int *active, cudaStream_t st) {
    if (nparts <= 0) return;
    gtau_kernel<<<dim3(grid_x(max_elems), nparts), kThreads, 0, st>>>(d, active);
    CCSD_LAUNCH_CHECK();
}

void launch_grouped_theta(const GAmp *d, int nparts, size_t max_elems, const int *active, cudaStream_t st) {
    if (nparts <= 0) return;
    gtheta_kernel<<<dim3(grid_x(max_elems), nparts), kThreads, 0, st>>>(d, active);
    CCSD_LAUNCH_CHECK();
}

void launch_grouped_tau_sym(const GAmp *d, int nparts, size_t max_elems, const int *active, cudaStream_t st) {
    if (nparts <= 0) return;
    gtau_sym_kernel<<<dim3(grid_x(max_elems), nparts), kThreads, 0, st>>>(d, active);
    CCSD_LAUNCH_CHECK();
}

void launch_grouped_unpack(const GAmp *d, int nparts, size_t max_elems, const int *active, cudaStream_t st) {
    if (nparts <= 0) return;
    gunpack_kernel<<<dim3(grid_x(max_elems), nparts), kThreads, 0, st>>>(d, active);
    CCSD_LAUNCH_CHECK();
}

int grouped_partials_per_part() { return kPer; }

void launch_grouped_update(const GUpdate *d, int nparts, const int *active, double *partials, cudaStream_t st) {
    if (nparts <= 0) return;
    gupdate_kernel<<<dim3(kUpdBlocks + 1, nparts), kThreads, 0, st>>>(d, active, partials);
    CCSD_LAUNCH_CHECK();
}

void launch_grouped_dot(const GDot *d, int nparts, const int *active, double *partials, cudaStream_t st) {
    if (nparts <= 0) return;
    gdot_kernel<<<dim3(kUpdBlocks + 1, nparts), kThreads, 0, st>>>(d, active, partials);
    CCSD_LAUNCH_CHECK();
}

void launch_grouped_sum(int nparts, const int *active, const double *partials, double *out, cudaStream_t st) {
    if (nparts <= 0) return;
    gsum_kernel<<<nparts, 32, 0, st>>>(active, partials, out);
    CCSD_LAUNCH_CHECK();
}

}  // namespace ccsd
