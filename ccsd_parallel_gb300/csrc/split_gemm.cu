// Split-precision contraction engine on the sm_103a tensor cores (tcgen05).
//
// Operands (split_gemm.h): S BF16 planes per FP64 operand row, K-major,
// per-row power-of-two scale.  Kernel: one 128 x BN output tile per CTA,
// warp-specialised:
//   warp 0      TMA producer: S planes of A (128 x 32) and of B (BN x 32) per
//               pipeline stage, 64-byte swizzle, one mbarrier per stage
//   warp 1      TMEM owner + single-thread tcgen05.mma issuer:
//                 level 0 (P0 x P0)  -> TMEM acc0[buf] (double-buffered),
//                                       restarted every 1024 K elements
//                 levels 1..S-1      -> TMEM rest (one FP32 accumulator)
//   warps 2..5  epilogue: drain acc0 after each 1024-K chunk into 32-bit
//               integer registers (the chunk sums are integers < 2^24, exact
//               in FP32), then C = alpha*sA*sB*2^-14*(I0 + rest) + beta*C.
// Every mbarrier wait is bounded in wall time; a wait that gives up sets a
// bit in the device error word, the other roles stop, in-flight TMA loads and
// MMAs are awaited (bounded) and TMEM is freed before the CTA exits.
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstring>
#include <string>

#include "../../include/ccsd_gb300.h"
#include "ptx.cuh"
#include "split_gemm.h"

namespace ccsd {

namespace {

constexpr int BM = 128;                  // MMA M (one CTA, cta_group::1)
constexpr int BK = 32;                   // K elements per stage (64 B rows)
constexpr int CHUNK_KB = 1024 / BK;      // k-blocks per exact level-0 chunk
constexpr int kThreads = 192;
constexpr uint64_t kWaitNs = 4000000000ull;  // 4 s wall-time bound per wait
constexpr int kMaxKbPerSplit = 131072 / BK;  // int32 level-0 sum stays < 2^31
constexpr int kGroupM = 16;                  // row tiles per rasterisation group

__host__ __device__ constexpr int stage_bytes(int S, int BN) { return S * (BM + BN) * BK * 2; }
__host__ __device__ constexpr int num_stages(int S, int BN) {
    return (220 * 1024) / stage_bytes(S, BN) < 8 ? (220 * 1024) / stage_bytes(S, BN) : 8;
}
__host__ __device__ constexpr int tmem_cols(int BN) {
    return 3 * BN <= 128 ? 128 : (3 * BN <= 256 ? 256 : 512);
}

struct alignas(8) Bars {
    uint64_t full[8];
    uint64_t empty[8];
    uint64_t acc_full[2];
    uint64_t acc_empty[2];
    uint64_t rest_full;
    uint64_t drain;
    uint32_t tmem_base;
    int abort;
    int never;  // stays 0: a wait that must not be cut short by another role
    int eb_min, eb_max;  // range of the tile's column-scale exponents (FP32 epilogue check)
};

// Behind the barriers: the tile's output column offsets and column scales, set
// once by the epilogue warps instead of per element (a 3-level column view costs
// tens of integer instructions per offset).
__host__ __device__ constexpr size_t epi_offset() { return (sizeof(Bars) + 15) / 16 * 16; }
__host__ __device__ constexpr size_t epi_bytes(int BN) {
    return (size_t)BN * (sizeof(int64_t) + sizeof(double) + sizeof(float));
}

// Binary exponent of a normal double (|x| in [2^e, 2^(e+1))); zero gives -1023.
__device__ __forceinline__ int exp2_of(double x) {
    return (int)((__double_as_longlong(x) >> 52) & 0x7FF) - 1023;
}

// The FP32 epilogue (S <= 3) forms (I0 + F) * sA * sB * alpha in FP32 and
// leaves one conversion and one FMA per element on the FP64 pipe, which runs
// at 1/64 of the FP32 rate on this part.  Rounding the sum to FP32 adds at most
// 2^-23 of |C_mn|, below split3's bound 2^-21 max|A_m| max|B_n| K.  A warp
// whose scale products could leave [2^-100, 2^90] (so that a sum below 2^32
// might overflow or a result become subnormal) keeps the FP64 epilogue.
constexpr int kEpi32Lo = -100, kEpi32Hi = 90;

// Failure injection (ccsd_debug_stall_split_mma): while non-zero, the MMA
// thread of every CTA first waits on an mbarrier that no role arrives at before
// its main loop (the drain barrier, whose first arrival is the final commit),
// bounded by this many nanoseconds.  The wait gives up and the CTA leaves
// through the time-out path of a real stall.
__device__ unsigned long long g_stall_mma_ns = 0;

}  // namespace

// What one CTA computes: a 128 x BN output tile of one contraction.  Rows of
// the tile's A (B) operand start at plane row rowA0 + mt*128 (rowB0 + nt*BN).
struct TileJob {
    int rowA0, rowB0;    // first plane row of the contraction's A / B operand
    int mt, nt;          // tile indices
    int M, N;            // C bounds
    int kb0, nkb;        // k-block range (32 K elements per block)
    const double *scaleA, *scaleB;  // row scales, indexed by the C row / column
    double alpha, beta;
    OutView C;
    double *wsz;  // split-K: partial-sum slab [M][N], else null (write C)
    bool run;
    bool c32;     // every column offset of C below 2^31 (the epilogue's offsets in 32 bits)
};

// One contraction over the whole grid (grouped rasterisation, split-K over z).
struct SingleJobs {
    int M, N, tiles_m, tiles_n, nkb_total, kb_per_split, splits;
    const double *scaleA, *scaleB;
    double alpha, beta;
    OutView C;
    double *ws;
    bool c32 = false;
    __device__ TileJob job() const { return at(blockIdx.x, blockIdx.z); }
    // Work item w of the persistent kernel: split-K slice z = w / tiles, tile w % tiles.
    __device__ TileJob job_at(int w) const {
        const int tiles = tiles_m * tiles_n, z = w / tiles;
        return at(w - z * tiles, z);
    }
    __device__ TileJob at(int t, int z) const {
        TileJob J;
        // Grouped rasterisation: consecutive CTAs walk kGroupM row tiles across
        // all column tiles, so the CTAs resident together share A and B tiles in L2.
        const int group = kGroupM * tiles_n;
        const int g = t / group, first_m = g * kGroupM;
        const int gm = min(tiles_m - first_m, kGroupM);
        const int local = t - g * group;
        J.mt = first_m + local % gm;
        J.nt = local / gm;
        J.rowA0 = J.rowB0 = 0;
        J.M = M;
        J.N = N;
        J.kb0 = z * kb_per_split;
        J.nkb = min(nkb_total, J.kb0 + kb_per_split) - J.kb0;
        J.scaleA = scaleA;
        J.scaleB = scaleB;
        J.alpha = alpha;
        J.beta = beta;
        J.c32 = c32;
        J.C = C;
        J.wsz = splits == 1 ? nullptr : ws + (size_t)z * M * N;
        J.run = true;
        return J;
    }
};

// Many systems' shares of one contraction (batched solve): part p's rows sit
// at rowA0 / rowB0 of packed plane buffers with a common row pitch; a CTA
// finds its part by binary search over the parts' first tiles.
struct GroupedJobs {
    const GroupedSplitPart *parts;
    int nparts;
    const int *active;
    __device__ TileJob job() const {
        TileJob J;
        const int t = blockIdx.x;
        int lo = 0, hi = nparts - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (parts[mid].tile_begin <= t) lo = mid;
            else hi = mid - 1;
        }
        const GroupedSplitPart &P = parts[lo];
        J.run = active[P.sys] != 0;
        const int local = t - P.tile_begin;
        J.mt = local % P.tiles_m;
        J.nt = local / P.tiles_m;
        J.rowA0 = P.rowA0;
        J.rowB0 = P.rowB0;
        J.M = P.M;
        J.N = P.N;
        J.kb0 = 0;
        J.nkb = P.nkb;
        J.scaleA = P.scaleA;
        J.scaleB = P.scaleB;
        J.alpha = P.alpha;
        J.beta = P.beta;
        J.C = P.C;
        J.wsz = nullptr;
        return J;
    }
};

namespace {

// NSTF: pipeline stages (0 = as many as fit one CTA per SM); MINB: CTAs per SM.
// Jobs: SingleJobs (one contraction) or GroupedJobs (one per system).
template <int S, int BN, int NSTF, int MINB, class Jobs>
__global__ void __launch_bounds__(kThreads, MINB)
    split_gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                      int rowsA_pad, int rowsB_pad, const Jobs jobs, int *gerr) {
    constexpr int NST = NSTF > 0 ? NSTF : num_stages(S, BN);
    constexpr int SB = stage_bytes(S, BN);
    constexpr int A_TILE = BM * BK * 2;   // bytes per A plane tile
    constexpr int B_TILE = BN * BK * 2;
    constexpr uint32_t IDESC = ptx::idesc_bf16_f32(BM, BN);
    constexpr int NCOLS = tmem_cols(BN);

    const TileJob J = jobs.job();
    if (!J.run) return;  // a stopped system: the whole CTA leaves before any set-up

    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char *smem = (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    Bars *bars = (Bars *)(smem + NST * SB);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = J.mt * BM, n0 = J.nt * BN, M = J.M, N = J.N;
    const int tma_m0 = J.rowA0 + m0, tma_n0 = J.rowB0 + n0;
    const int kb0 = J.kb0;
    const int nkb = J.nkb;
    const int nch = (nkb + CHUNK_KB - 1) / CHUNK_KB;
    const double *__restrict__ scaleA = J.scaleA;
    const double *__restrict__ scaleB = J.scaleB;
    const double alpha = J.alpha, beta = J.beta;
    const OutView C = J.C;
    const bool rdc = J.wsz == nullptr && beta != 0.0;  // reads C (one FP64 comparison)

    if (threadIdx.x == 0) {
        for (int s = 0; s < NST; ++s) {
            ptx::mbar_init(&bars->full[s], 1);
            ptx::mbar_init(&bars->empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            ptx::mbar_init(&bars->acc_full[b], 1);
            ptx::mbar_init(&bars->acc_empty[b], 4);
        }
        ptx::mbar_init(&bars->rest_full, 1);
        ptx::mbar_init(&bars->drain, 1);
        bars->abort = 0;
        bars->never = 0;
        bars->eb_min = 1 << 20;
        bars->eb_max = -(1 << 20);
        ptx::fence_barrier_init();
        ptx::prefetch_tmap(&tmA);
        ptx::prefetch_tmap(&tmB);
    }
    if (warp == 1) {
        ptx::tmem_alloc(&bars->tmem_base, NCOLS);
        ptx::tmem_relinquish();
    }
    ptx::tc_fence_before();
    __syncthreads();
    ptx::tc_fence_after();
    const uint32_t tmem = bars->tmem_base;
    volatile int *abort = &bars->abort;

    if (warp == 0) {
        if (lane == 0 && nkb > 0) {
            int issued = 0;
            for (int l = 0; l < nkb; ++l) {
                const int st = l % NST, round = l / NST;
                if (!ptx::mbar_wait(&bars->empty[st], (round & 1) ^ 1, abort, gerr, 1, kWaitNs)) break;
                ptx::mbar_arrive_expect_tx(&bars->full[st], SB);
                unsigned char *sa = smem + st * SB;
                unsigned char *sb = sa + S * A_TILE;
                const int kx = (kb0 + l) * BK;
#pragma unroll
                for (int p = 0; p < S; ++p) {
                    ptx::tma_load_2d(sa + p * A_TILE, &tmA, &bars->full[st], kx, p * rowsA_pad + tma_m0);
                    ptx::tma_load_2d(sb + p * B_TILE, &tmB, &bars->full[st], kx, p * rowsB_pad + tma_n0);
                }
                issued = l + 1;
            }
            if (*abort) {  // let every TMA load this thread issued land before the CTA exits
                for (int l = max(0, issued - NST); l < issued; ++l)
                    ptx::mbar_wait(&bars->full[l % NST], (l / NST) & 1, &bars->never, gerr, 2, kWaitNs);
            }
        }
    } else if (warp == 1) {
        if (lane == 0 && nkb > 0) {
            const unsigned long long stall = g_stall_mma_ns;
            const bool go = stall == 0 || ptx::mbar_wait(&bars->drain, 0, abort, gerr, 128, stall);
            bool first_rest = true;
            for (int l = 0; go && l < nkb; ++l) {
                const int st = l % NST, round = l / NST;
                const int c = l / CHUNK_KB, b = c & 1;
                const bool chunk_start = (l % CHUNK_KB) == 0;
                if (chunk_start) {
                    if (!ptx::mbar_wait(&bars->acc_empty[b], ((c >> 1) & 1) ^ 1, abort, gerr, 4, kWaitNs)) break;
                    ptx::tc_fence_after();
                }
                if (!ptx::mbar_wait(&bars->full[st], round & 1, abort, gerr, 8, kWaitNs)) break;
                ptx::tc_fence_after();
                const uint32_t sa = ptx::smem_u32(smem + st * SB);
                const uint32_t sb = sa + S * A_TILE;
#pragma unroll
                for (int kk = 0; kk < BK / 16; ++kk) {
                    uint64_t ad[S], bd[S];
#pragma unroll
                    for (int p = 0; p < S; ++p) {
                        ad[p] = ptx::sdesc_k_sw64(sa + p * A_TILE + kk * 32);
                        bd[p] = ptx::sdesc_k_sw64(sb + p * B_TILE + kk * 32);
                    }
                    ptx::mma_bf16(tmem + b * BN, ad[0], bd[0], IDESC, (chunk_start && kk == 0) ? 0u : 1u);
#pragma unroll
                    for (int lev = 1; lev < S; ++lev)
#pragma unroll
                        for (int p = 0; p <= lev; ++p) {
                            ptx::mma_bf16(tmem + 2 * BN, ad[p], bd[lev - p], IDESC, first_rest ? 0u : 1u);
                            first_rest = false;
                        }
                }
                ptx::mma_commit(&bars->empty[st]);
                if ((l % CHUNK_KB) == CHUNK_KB - 1 || l == nkb - 1) ptx::mma_commit(&bars->acc_full[b]);
            }
            ptx::mma_commit(&bars->rest_full);
            ptx::mma_commit(&bars->drain);
            ptx::mbar_wait(&bars->drain, 0, &bars->never, gerr, 16, kWaitNs);
        }
    } else {
        // epilogue warps 2..5; TMEM lane quarter = warp % 4
        const int q = warp & 3;
        const uint32_t lane_off = (uint32_t)(q * 32) << 16;
        int64_t *s_coff = (int64_t *)((unsigned char *)bars + epi_offset());
        double *s_sb = (double *)(s_coff + BN);
        float *s_fsb = (float *)(s_sb + BN);
        constexpr bool kEpi32 = S <= 3;
        for (int j = threadIdx.x - 64; j < BN; j += 128) {
            const int n = n0 + j;
            const double sbn = n < N ? scaleB[n] : 0.0;
            s_coff[j] = n < N ? dim_off(C.col, (uint32_t)n) : -1;
            s_sb[j] = sbn;
            if (kEpi32) {
                s_fsb[j] = (float)sbn;
                if (n < N) {
                    const int e = exp2_of(sbn);
                    atomicMin(&bars->eb_min, e);
                    atomicMax(&bars->eb_max, e);
                }
            }
        }
        asm volatile("bar.sync 1, 128;" ::: "memory");  // the four epilogue warps only
        int32_t iacc[BN];
#pragma unroll
        for (int j = 0; j < BN; ++j) iacc[j] = 0;
        bool ok = nkb > 0;
        for (int c = 0; c < nch && ok; ++c) {
            const int b = c & 1;
            const bool got = ptx::mbar_wait(&bars->acc_full[b], (c >> 1) & 1, abort, gerr, 32, kWaitNs);
            if (!__all_sync(0xffffffffu, got)) {  // keep the warp converged for tcgen05.ld
                ok = false;
                break;
            }
            ptx::tc_fence_after();
#pragma unroll
            for (int g = 0; g < BN / 32; ++g) {
                uint32_t r[32];
                ptx::tmem_ld32(tmem + lane_off + b * BN + g * 32, r);
                ptx::tmem_ld_wait();
#pragma unroll
                for (int j = 0; j < 32; ++j) iacc[g * 32 + j] += __float2int_rn(__uint_as_float(r[j]));
            }
            ptx::tc_fence_before();
            __syncwarp();
            if (lane == 0) ptx::mbar_arrive(&bars->acc_empty[b]);
        }
        if (ok) ok = __all_sync(0xffffffffu, ptx::mbar_wait(&bars->rest_full, 0, abort, gerr, 64, kWaitNs));
        if (ok || nkb == 0) {
            ptx::tc_fence_after();
            const int m = m0 + q * 32 + lane;
            const bool mval = m < M;
            const double sa = mval ? scaleA[m] * 0x1.0p-14 : 0.0;
            const int64_t crow = mval ? dim_off(C.row, (uint32_t)m) : 0;
            const bool direct = J.wsz == nullptr;
            double *wsz = J.wsz;
            // FP32 epilogue: the row factor sa (times alpha when writing C) as a float, if
            // every scale product of this warp's rows stays in range
            const double sa_out = direct ? sa * alpha : sa;
            const int ea = exp2_of(sa_out);
            const bool in_range = !mval || sa_out == 0.0 ||
                                  (ea + bars->eb_min >= kEpi32Lo && ea + bars->eb_max <= kEpi32Hi);
            const bool epi32 = kEpi32 && __all_sync(0xffffffffu, in_range);
            const float fsa = (float)sa_out;
#pragma unroll
            for (int g = 0; g < BN / 32; ++g) {
                uint32_t r[32];
                if (nkb > 0) {
                    ptx::tmem_ld32(tmem + lane_off + 2 * BN + g * 32, r);
                    ptx::tmem_ld_wait();
                } else {
#pragma unroll
                    for (int j = 0; j < 32; ++j) r[j] = 0u;
                }
                // kCB columns at a time: their C loads (beta != 0) are issued
                // together instead of one dependent load per column
                constexpr int kCB = 4;
#pragma unroll
                for (int j0 = 0; j0 < 32; j0 += kCB) {
                    int64_t off[kCB];
                    double cold[kCB];
#pragma unroll
                    for (int j = 0; j < kCB; ++j) {
                        const int64_t co = s_coff[g * 32 + j0 + j];
                        off[j] = (mval && co >= 0) ? crow + co : -1;
                        cold[j] = (rdc && off[j] >= 0) ? C.p[off[j]] : 0.0;
                    }
#pragma unroll
                    for (int j = 0; j < kCB; ++j) {
                        if (off[j] < 0) continue;
                        const int n = n0 + g * 32 + j0 + j;
                        const int jj = g * 32 + j0 + j;
                        if (kEpi32 && epi32) {
                            const float f = (__int2float_rn(iacc[jj]) + __uint_as_float(r[j0 + j])) * fsa *
                                            s_fsb[jj];
                            const double val = (double)f;
                            if (direct)
                                C.p[off[j]] = rdc ? fma(beta, cold[j], val) : val;
                            else
                                wsz[(size_t)m * N + n] = val;
                            continue;
                        }
                        const double val = sa * s_sb[jj] * ((double)iacc[jj] + (double)__uint_as_float(r[j0 + j]));
                        if (direct) {
                            double out = alpha * val;
                            if (rdc) out = fma(beta, cold[j], out);
                            C.p[off[j]] = out;
                        } else {
                            wsz[(size_t)m * N + n] = val;
                        }
                    }
                }
            }
        }
    }

    ptx::tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        ptx::tc_fence_after();
        ptx::tmem_dealloc(tmem, NCOLS);
    }
}

// ---- persistent form of one contraction ------------------------------------
// A CTA walks the work items w = blockIdx.x, blockIdx.x + gridDim.x, ... (tiles
// in the grouped order, split-K slices folded in).  The producer streams the
// k-blocks of consecutive tiles through the stage ring without draining it, and
// the accumulators are arranged so that a tile's epilogue runs while the MMA
// issuer works on the next tile: the level-0 chunk buffers acc0[0..1] alternate
// over the chunk count of all the CTA's tiles, and the higher levels get one
// buffer per tile parity, rest[0..1].  TMEM columns: acc0[0], acc0[1], rest[0],
// rest[1], BN each.  The epilogue warps keep private column tables, so no
// barrier spans warps inside the tile loop and every wait stays bounded.
struct PBars {
    uint64_t full[8];
    uint64_t empty[8];
    uint64_t acc_full[2];
    uint64_t acc_empty[2];
    uint64_t rest_full[2];
    uint64_t rest_empty[2];
    uint64_t drain;
    uint32_t tmem_base;
    int abort;
    int never;
};
__host__ __device__ constexpr size_t pbars_bytes() { return (sizeof(PBars) + 15) / 16 * 16; }
__host__ __device__ constexpr int ptmem_cols(int BN) { return 4 * BN <= 128 ? 128 : (4 * BN <= 256 ? 256 : 512); }

// EW epilogue warps (warps 2 .. EW+1): warp w covers TMEM lane quarter w % 4 and the
// column slice (w - 2) / 4 of BN / (EW / 4) columns; KCB C loads are issued together.
template <int S, int BN, int NST, int MINB, int EW, int KCB>
__global__ void __launch_bounds__(64 + 32 * EW, MINB)
    split_gemm_persistent_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                                 int rowsA_pad, int rowsB_pad, const SingleJobs jobs, int nwork, int *gerr) {
    constexpr int SB = stage_bytes(S, BN);
    constexpr int A_TILE = BM * BK * 2;
    constexpr int B_TILE = BN * BK * 2;
    constexpr uint32_t IDESC = ptx::idesc_bf16_f32(BM, BN);
    constexpr int NCOLS = ptmem_cols(BN);
    constexpr bool kEpi32 = S <= 3;
    static_assert(4 * BN <= 512, "four BN-column accumulators must fit in TMEM");
    static_assert(EW == 4 || EW == 8, "four or eight epilogue warps");
    constexpr int BW = BN / (EW / 4);  // columns per epilogue warp
    static_assert(BW % 32 == 0 && 32 % KCB == 0, "column slices of whole 32-column groups");

    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char *smem = (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    PBars *bars = (PBars *)(smem + NST * SB);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    if (threadIdx.x == 0) {
        for (int st = 0; st < NST; ++st) {
            ptx::mbar_init(&bars->full[st], 1);
            ptx::mbar_init(&bars->empty[st], 1);
        }
        for (int b = 0; b < 2; ++b) {
            ptx::mbar_init(&bars->acc_full[b], 1);
            ptx::mbar_init(&bars->acc_empty[b], EW);
            ptx::mbar_init(&bars->rest_full[b], 1);
            ptx::mbar_init(&bars->rest_empty[b], EW);
        }
        ptx::mbar_init(&bars->drain, 1);
        bars->abort = 0;
        bars->never = 0;
        ptx::fence_barrier_init();
        ptx::prefetch_tmap(&tmA);
        ptx::prefetch_tmap(&tmB);
    }
    if (warp == 1) {
        ptx::tmem_alloc(&bars->tmem_base, NCOLS);
        ptx::tmem_relinquish();
    }
    ptx::tc_fence_before();
    __syncthreads();
    ptx::tc_fence_after();
    const uint32_t tmem = bars->tmem_base;
    volatile int *abort = &bars->abort;

    if (warp == 0) {
        if (lane == 0) {
            int g = 0, issued = 0;
            bool stop = false;
            for (int w = blockIdx.x; w < nwork && !stop; w += gridDim.x) {
                const TileJob J = jobs.job_at(w);
                const int tma_m0 = J.mt * BM, tma_n0 = J.nt * BN;
                for (int l = 0; l < J.nkb; ++l, ++g) {
                    const int st = g % NST, round = g / NST;
                    if (!ptx::mbar_wait(&bars->empty[st], (round & 1) ^ 1, abort, gerr, 1, kWaitNs)) {
                        stop = true;
                        break;
                    }
                    ptx::mbar_arrive_expect_tx(&bars->full[st], SB);
                    unsigned char *sa = smem + st * SB;
                    unsigned char *sb = sa + S * A_TILE;
                    const int kx = (J.kb0 + l) * BK;
#pragma unroll
                    for (int p = 0; p < S; ++p) {
                        ptx::tma_load_2d(sa + p * A_TILE, &tmA, &bars->full[st], kx, p * rowsA_pad + tma_m0);
                        ptx::tma_load_2d(sb + p * B_TILE, &tmB, &bars->full[st], kx, p * rowsB_pad + tma_n0);
                    }
                    issued = g + 1;
                }
            }
            if (*abort) {  // let every TMA load this thread issued land before the CTA exits
                for (int l = max(0, issued - NST); l < issued; ++l)
                    ptx::mbar_wait(&bars->full[l % NST], (l / NST) & 1, &bars->never, gerr, 2, kWaitNs);
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            const unsigned long long stall = g_stall_mma_ns;
            bool ok = stall == 0 || ptx::mbar_wait(&bars->drain, 0, abort, gerr, 128, stall);
            int g = 0, c = 0, n = 0;
            for (int w = blockIdx.x; w < nwork && ok; w += gridDim.x, ++n) {
                const TileJob J = jobs.job_at(w);
                const int j = n & 1;
                // rest[j] is free once the epilogue of tile n - 2 has read it
                if (!ptx::mbar_wait(&bars->rest_empty[j], ((n >> 1) & 1) ^ 1, abort, gerr, 4, kWaitNs)) {
                    ok = false;
                    break;
                }
                ptx::tc_fence_after();
                const uint32_t rest = tmem + (2 + j) * BN;
                bool first_rest = true;
                for (int l = 0; l < J.nkb; ++l, ++g) {
                    const int st = g % NST, round = g / NST;
                    const int b = c & 1;
                    const bool chunk_start = (l % CHUNK_KB) == 0;
                    if (chunk_start) {
                        if (!ptx::mbar_wait(&bars->acc_empty[b], ((c >> 1) & 1) ^ 1, abort, gerr, 4, kWaitNs)) {
                            ok = false;
                            break;
                        }
                        ptx::tc_fence_after();
                    }
                    if (!ptx::mbar_wait(&bars->full[st], round & 1, abort, gerr, 8, kWaitNs)) {
                        ok = false;
                        break;
                    }
                    ptx::tc_fence_after();
                    const uint32_t sa = ptx::smem_u32(smem + st * SB);
                    const uint32_t sb = sa + S * A_TILE;
#pragma unroll
                    for (int kk = 0; kk < BK / 16; ++kk) {
                        uint64_t ad[S], bd[S];
#pragma unroll
                        for (int p = 0; p < S; ++p) {
                            ad[p] = ptx::sdesc_k_sw64(sa + p * A_TILE + kk * 32);
                            bd[p] = ptx::sdesc_k_sw64(sb + p * B_TILE + kk * 32);
                        }
                        ptx::mma_bf16(tmem + b * BN, ad[0], bd[0], IDESC, (chunk_start && kk == 0) ? 0u : 1u);
#pragma unroll
                        for (int lev = 1; lev < S; ++lev)
#pragma unroll
                            for (int p = 0; p <= lev; ++p) {
                                ptx::mma_bf16(rest, ad[p], bd[lev - p], IDESC, first_rest ? 0u : 1u);
                                first_rest = false;
                            }
                    }
                    ptx::mma_commit(&bars->empty[st]);
                    if ((l % CHUNK_KB) == CHUNK_KB - 1 || l == J.nkb - 1) {
                        ptx::mma_commit(&bars->acc_full[b]);
                        ++c;
                    }
                }
                if (!ok) break;
                ptx::mma_commit(&bars->rest_full[j]);
            }
            ptx::mma_commit(&bars->drain);
            ptx::mbar_wait(&bars->drain, 0, &bars->never, gerr, 16, kWaitNs);
        }
    } else {
        // epilogue warps 2 .. EW+1; TMEM lane quarter = warp % 4, column slice (warp - 2) / 4;
        // each warp keeps its own column table (offsets, FP64 and FP32 column scales)
        const int q = warp & 3;
        const int c0 = ((warp - 2) >> 2) * BW;  // first column of this warp's slice
        const uint32_t lane_off = (uint32_t)(q * 32) << 16;
        unsigned char *tbl = (unsigned char *)bars + pbars_bytes() + (size_t)(warp - 2) * epi_bytes(BW);
        int64_t *s_coff = (int64_t *)tbl;
        double *s_sb = (double *)(s_coff + BW);
        float *s_fsb = (float *)(s_sb + BW);
        int c = 0, n = 0;
        for (int w = blockIdx.x; w < nwork; w += gridDim.x, ++n) {
            const TileJob J = jobs.job_at(w);
            const int j = n & 1;
            const int m0 = J.mt * BM, n0 = J.nt * BN + c0, M = J.M, N = J.N, nkb = J.nkb;
            const OutView C = J.C;
            __syncwarp();  // the previous tile's table reads are done
            int ebmin = 1 << 20, ebmax = -(1 << 20);
            for (int jj = lane; jj < BW; jj += 32) {
                const int nn = n0 + jj;
                const double sbn = nn < N ? J.scaleB[nn] : 0.0;
                const int64_t co = nn < N ? dim_off(C.col, (uint32_t)nn) : -1;
                if (J.c32)
                    reinterpret_cast<int32_t *>(s_coff)[jj] = (int32_t)co;
                else
                    s_coff[jj] = co;
                s_sb[jj] = sbn;
                s_fsb[jj] = (float)sbn;
                if (nn < N) {
                    const int e = exp2_of(sbn);
                    ebmin = min(ebmin, e);
                    ebmax = max(ebmax, e);
                }
            }
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                ebmin = min(ebmin, __shfl_xor_sync(0xffffffffu, ebmin, off));
                ebmax = max(ebmax, __shfl_xor_sync(0xffffffffu, ebmax, off));
            }
            __syncwarp();
            int32_t iacc[BW];
#pragma unroll
            for (int jj = 0; jj < BW; ++jj) iacc[jj] = 0;
            const int nch = (nkb + CHUNK_KB - 1) / CHUNK_KB;
            bool ok = true;
            for (int ch = 0; ch < nch; ++ch, ++c) {
                const int b = c & 1;
                const bool got = ptx::mbar_wait(&bars->acc_full[b], (c >> 1) & 1, abort, gerr, 32, kWaitNs);
                if (!__all_sync(0xffffffffu, got)) {  // keep the warp converged for tcgen05.ld
                    ok = false;
                    break;
                }
                ptx::tc_fence_after();
#pragma unroll
                for (int gq = 0; gq < BW / 32; ++gq) {
                    uint32_t r[32];
                    ptx::tmem_ld32(tmem + lane_off + b * BN + c0 + gq * 32, r);
                    ptx::tmem_ld_wait();
#pragma unroll
                    for (int jj = 0; jj < 32; ++jj) iacc[gq * 32 + jj] += __float2int_rn(__uint_as_float(r[jj]));
                }
                ptx::tc_fence_before();
                __syncwarp();
                if (lane == 0) ptx::mbar_arrive(&bars->acc_empty[b]);
            }
            if (ok) ok = __all_sync(0xffffffffu, ptx::mbar_wait(&bars->rest_full[j], (n >> 1) & 1, abort, gerr, 64, kWaitNs));
            if (!ok) break;
            ptx::tc_fence_after();
            const int m = m0 + q * 32 + lane;
            const bool mval = m < M;
            const double sa = mval ? J.scaleA[m] * 0x1.0p-14 : 0.0;
            const int64_t crow = mval ? dim_off(C.row, (uint32_t)m) : 0;
            const bool direct = J.wsz == nullptr;
            double *wsz = J.wsz;
            const double alpha = J.alpha, beta = J.beta;
            const bool rdc = direct && beta != 0.0;  // reads C (one FP64 comparison per tile)
            const double sa_out = direct ? sa * alpha : sa;
            const int ea = exp2_of(sa_out);
            const bool in_range = !mval || sa_out == 0.0 || (ea + ebmin >= kEpi32Lo && ea + ebmax <= kEpi32Hi);
            const bool epi32 = kEpi32 && __all_sync(0xffffffffu, in_range);
            const float fsa = (float)sa_out;
            const uint32_t rest = tmem + (2 + j) * BN + c0;
            double *cb = C.p + crow;  // this lane's row of C; columns at cb + offset
            // the element loop over 32- or 64-bit column offsets (64-bit integer arithmetic
            // issues on the FP64 pipe on this part, which the epilogue's FMA also needs)
            auto drain = [&](auto zero) {
                using OffT = decltype(zero);
                const OffT *coff = reinterpret_cast<const OffT *>(s_coff);
#pragma unroll
                for (int gq = 0; gq < BW / 32; ++gq) {
                    uint32_t r[32];
                    ptx::tmem_ld32(rest + lane_off + gq * 32, r);
                    ptx::tmem_ld_wait();
#pragma unroll
                    for (int j0 = 0; j0 < 32; j0 += KCB) {
                        OffT off[KCB];
                        double cold[KCB];
#pragma unroll
                        for (int u = 0; u < KCB; ++u) {
                            const OffT co = coff[gq * 32 + j0 + u];
                            off[u] = mval ? co : (OffT)-1;
                            cold[u] = (rdc && off[u] >= 0) ? cb[off[u]] : 0.0;
                        }
#pragma unroll
                        for (int u = 0; u < KCB; ++u) {
                            if (off[u] < 0) continue;
                            const int nn = n0 + gq * 32 + j0 + u;
                            const int jj = gq * 32 + j0 + u;
                            if (kEpi32 && epi32) {
                                const float f =
                                    (__int2float_rn(iacc[jj]) + __uint_as_float(r[j0 + u])) * fsa * s_fsb[jj];
                                const double val = (double)f;
                                if (direct)
                                    cb[off[u]] = rdc ? fma(beta, cold[u], val) : val;
                                else
                                    wsz[(size_t)m * N + nn] = val;
                                continue;
                            }
                            const double val =
                                sa * s_sb[jj] * ((double)iacc[jj] + (double)__uint_as_float(r[j0 + u]));
                            if (direct) {
                                double out = alpha * val;
                                if (rdc) out = fma(beta, cold[u], out);
                                cb[off[u]] = out;
                            } else {
                                wsz[(size_t)m * N + nn] = val;
                            }
                        }
                    }
                }
            };
            if (J.c32)
                drain(int32_t(0));
            else
                drain(int64_t(0));
            ptx::tc_fence_before();
            __syncwarp();
            if (lane == 0) ptx::mbar_arrive(&bars->rest_empty[j]);
        }
    }

    ptx::tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        ptx::tc_fence_after();
        ptx::tmem_dealloc(tmem, NCOLS);
    }
}

// ---- FP64 -> S BF16 planes ---------------------------------------------------
// All integer arithmetic (FP64 runs at 1/64 of the FP32 rate on this part):
// pass 1 takes the row maxima of |x| as the high words of their IEEE bit patterns
// (they order like the values' exponents for non-negative doubles); pass 2 turns x into the fixed-point
// integer Y = round(x * 2^(7 - ex + 8(S-1))), ex = exponent of the row
// maximum (|Y| <= 2^(8S-1)), and peels balanced base-256 digits
// d in [-128, 127] off Y from the bottom; the remaining top digit P0 lies in
// [-128, 128].  Plane p stores d_p * 2^(-8p), exact in BF16.
constexpr int kRowmaxKT = 32;  // 32-wide k tiles per row-max block

// Row maxima of one 32-row x (32 kRowmaxKT)-column block, from row r0 and
// column kbeg, merged into rmax with atomicMax (32 x 8 threads).  A row maximum
// is kept as the high word of |x| (sign cleared), which orders |x| by exponent:
// only the exponent is used, and the comparisons stay 32-bit (64-bit integer
// arithmetic issues on the FP64 pipe on this part).  Four loads per thread are
// issued before their maxima are taken.
template <bool ROWC>
__device__ void rowmax_block(int rows, int K, const MatView &v, unsigned long long *rmax, int r0, int kbeg) {
    const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
    const auto hiabs = [](double x) { return (uint32_t)__double2hiint(x) & 0x7FFFFFFFu; };
    if (ROWC) {
        // thread owns row r0 + tx; the 8 thread rows split the k range
        __shared__ uint32_t part[8][32];
        const int r = r0 + tx;
        uint32_t m = 0;
        if (r < rows) {
            const double *row = v.p + dim_off(v.row, (uint32_t)r);
            const int kend = min(K, kbeg + 32 * kRowmaxKT);
            int k = kbeg + ty;
            for (; k + 24 < kend; k += 32) {
                const double x0 = row[dim_off(v.col, (uint32_t)k)], x1 = row[dim_off(v.col, (uint32_t)(k + 8))];
                const double x2 = row[dim_off(v.col, (uint32_t)(k + 16))], x3 = row[dim_off(v.col, (uint32_t)(k + 24))];
                m = max(max(m, max(hiabs(x0), hiabs(x1))), max(hiabs(x2), hiabs(x3)));
            }
            for (; k < kend; k += 8) m = max(m, hiabs(row[dim_off(v.col, (uint32_t)k)]));
        }
        part[ty][tx] = m;
        __syncthreads();
        if (ty == 0 && r < rows) {
#pragma unroll
            for (int q = 1; q < 8; ++q) m = max(m, part[q][tx]);
            if (m) atomicMax(rmax + r, (unsigned long long)m);
        }
    } else {
        // thread row ty owns rows r0 + ty + 8j; lanes run along k
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int r = r0 + ty + 8 * j;
            uint32_t m = 0;
            if (r < rows) {
                const double *row = v.p + dim_off(v.row, (uint32_t)r);
                const int kend = min(K, kbeg + 32 * kRowmaxKT);
                int k = kbeg + tx;
                for (; k + 96 < kend; k += 128) {
                    const double x0 = row[dim_off(v.col, (uint32_t)k)], x1 = row[dim_off(v.col, (uint32_t)(k + 32))];
                    const double x2 = row[dim_off(v.col, (uint32_t)(k + 64))],
                                 x3 = row[dim_off(v.col, (uint32_t)(k + 96))];
                    m = max(max(m, max(hiabs(x0), hiabs(x1))), max(hiabs(x2), hiabs(x3)));
                }
                for (; k < kend; k += 32) m = max(m, hiabs(row[dim_off(v.col, (uint32_t)k)]));
            }
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, off));
            if (tx == 0 && r < rows && m) atomicMax(rmax + r, (unsigned long long)m);
        }
    }
    __syncthreads();  // the shared row maxima are reused by the next block of a looping caller
}

template <bool ROWC>
__global__ void rowmax_kernel(int rows, int K, int nkg, MatView v, unsigned long long *rmax) {
    rowmax_block<ROWC>(rows, K, v, rmax, (int)(blockIdx.x / nkg) * 32, (int)(blockIdx.x % nkg) * 32 * kRowmaxKT);
}

template <bool ROWC>
__device__ __forceinline__ void load_tile(double (&t)[32][33], int rows, int K, const MatView &v, int r0,
                                          int k0) {
    const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int a = ty + 8 * j;
        const int r = ROWC ? r0 + tx : r0 + a;
        const int k = ROWC ? k0 + a : k0 + tx;
        double x = 0.0;
        if (r < rows && k < K) x = v.p[dim_off(v.row, (uint32_t)r) + dim_off(v.col, (uint32_t)k)];
        if (ROWC)
            t[tx][a] = x;
        else
            t[a][tx] = x;
    }
}

// The S plane values of x for a row whose maximum has biased exponent emax
// (0 for a zero row): Y = round(x 2^(7 - e + 8(S-1))) as an integer, peeled into
// balanced base-256 digits from the bottom; plane p holds d_p 2^(-8p).  For S <= 3,
// |Y| <= 2^23 and the right shift is at least 30, so the digits are peeled in 32-bit
// integers and turned into floats by the exact 1.5 * 2^23 offset (an integer add and
// an FP32 subtract per digit); this runs on the integer and FP32 pipes only.
__device__ __forceinline__ float small_int_to_float(int32_t d) {  // exact for |d| < 2^22
    return __int_as_float(0x4B400000 + d) - 12582912.0f;
}

// A digit value d 2^(-8p) (|d| <= 128) has at most 8 significant bits, so its float
// encoding ends in 16 zero bits and the BF16 encoding is the top half: taken with
// integer byte moves instead of the conversion instruction (which issues on the
// FP64 pipe on this part).
__device__ __forceinline__ uint32_t bf16x2_of_digits(float lo, float hi) {
    return __byte_perm(__float_as_uint(lo), __float_as_uint(hi), 0x7632);
}
__device__ __forceinline__ __nv_bfloat16 bf16_of_digit(float f) {
    return __ushort_as_bfloat16((unsigned short)(__float_as_uint(f) >> 16));
}

template <int S>
__device__ __forceinline__ void split_digits(double x, int emax, float (&out)[S]) {
    const uint32_t hi = (uint32_t)__double2hiint(x), lo = (uint32_t)__double2loint(x);
    const int e = (int)((hi >> 20) & 0x7FF);
    const int rs = emax - e + 54 - 8 * S;  // right shift that puts x on the 2^-(8(S-1)) grid
    if constexpr (S <= 3) {
        // q = (mant + 2^(rs-1)) >> rs on the two 32-bit words of mant = mh 2^32 + lo
        // (rs >= 30; 64-bit integer arithmetic issues on the FP64 pipe here)
        int32_t Y = 0;
        if (emax && e && rs < 63) {
            const uint32_t mh = (hi & 0xFFFFFu) | 0x100000u;
            uint32_t q;
            if (rs >= 33) {  // the rounding bit lies in the high word; lo cannot carry past it
                q = (mh + (1u << (rs - 33))) >> (rs - 32);
            } else {
                const uint32_t l2 = lo + (1u << (rs - 1));
                const uint32_t h2 = mh + (l2 < lo ? 1u : 0u);
                q = rs == 32 ? h2 : __funnelshift_r(l2, h2, rs);
            }
            Y = (hi >> 31) ? -(int32_t)q : (int32_t)q;
        }
#pragma unroll
        for (int p = S - 1; p >= 1; --p) {
            const int32_t d = ((Y + 128) & 255) - 128;
            Y = (Y - d) >> 8;
            out[p] = small_int_to_float(d) * __int_as_float((127 - 8 * p) << 23);  // d 2^(-8p)
        }
        out[0] = small_int_to_float(Y);
    } else {
        const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
        long long Y = 0;
        if (emax && e && rs < 63) {
            const unsigned long long mant = (bits & 0xFFFFFFFFFFFFFull) | (1ull << 52);
            Y = (long long)((mant + (1ull << (rs - 1))) >> rs);
            if (bits >> 63) Y = -Y;
        }
#pragma unroll
        for (int p = S - 1; p >= 1; --p) {
            const long long d = ((Y + 128) & 255) - 128;
            Y = (Y - d) >> 8;
            out[p] = small_int_to_float((int32_t)d) * __int_as_float((127 - 8 * p) << 23);
        }
        out[0] = small_int_to_float((int32_t)Y);
    }
}

// Digits of one 32 x 32 block from row r0 and column k0.  Rows below rows_pad
// and columns below kpad are written (zeros past rows / K); row r of plane p
// sits at planes + p * plane + r * pitch.
template <int S, bool ROWC>
__device__ void planes_block(int rows, int rows_pad, int K, int kpad, int64_t pitch, size_t plane, const MatView &v,
                             const unsigned long long *rmax, __nv_bfloat16 *planes, double *scale, int r0, int k0) {
    __shared__ double t[32][33];
    load_tile<ROWC>(t, rows, K, v, r0, k0);
    __syncthreads();
    const int tx = threadIdx.x, ty = threadIdx.y;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int a = ty + 8 * j;
        const int r = r0 + a, k = k0 + tx;
        if (r >= rows_pad || k >= kpad) continue;
        const int emax = r < rows ? (int)((rmax[r] >> 20) & 0x7FF) : 0;  // 0: zero (or denormal) row
        if (k0 == 0 && tx == 0)
            scale[r] = emax ? __longlong_as_double((long long)(emax + 1) << 52) : 1.0;  // 2^(emax-1022)
        float d[S];
        split_digits<S>(t[a][tx], emax, d);
        __nv_bfloat16 *dst = planes + (size_t)r * pitch + k;
#pragma unroll
        for (int p = 0; p < S; ++p) dst[p * plane] = bf16_of_digit(d[p]);
    }
    __syncthreads();  // t is reused by the next block of a looping caller
}

// One pass for operands read along k: a warp owns a row, takes its maximum, then
// reads it again (from L2: one row at a time per warp) and writes its digits, two
// consecutive k per lane.  Rows past `rows` are not written: TMA boxes that run
// into them only feed output rows or columns the epilogue discards.  The K padding
// up to kpad is written as zeros (it enters every output).
template <int S>
__global__ void __launch_bounds__(256) split_rows_kernel(int rows, int K, int kpad, MatView v,
                                                         __nv_bfloat16 *__restrict__ planes, size_t plane,
                                                         double *__restrict__ scale) {
    const int lane = threadIdx.x & 31;
    const int warp = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    const int nwarps = (int)(((size_t)gridDim.x * blockDim.x) >> 5);
    const unsigned long long absmask = 0x7FFFFFFFFFFFFFFFull;
    for (int r = warp; r < rows; r += nwarps) {
        const int64_t ro = dim_off(v.row, (uint32_t)r);
        unsigned long long m = 0;
        for (int k = lane; k < K; k += 32) {
            const unsigned long long b =
                (unsigned long long)__double_as_longlong(v.p[ro + dim_off(v.col, (uint32_t)k)]) & absmask;
            m = b > m ? b : m;
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            const unsigned long long o2 = __shfl_xor_sync(0xffffffffu, m, off);
            m = o2 > m ? o2 : m;
        }
        const int emax = (int)((m >> 52) & 0x7FF);  // 0: zero (or denormal) row
        if (lane == 0) scale[r] = emax ? __longlong_as_double((long long)(emax + 1) << 52) : 1.0;
        __nv_bfloat16 *dst = planes + (size_t)r * kpad;
        for (int k = 2 * lane; k < kpad; k += 64) {
            float d0[S], d1[S];
            split_digits<S>(k < K ? v.p[ro + dim_off(v.col, (uint32_t)k)] : 0.0, emax, d0);
            split_digits<S>(k + 1 < K ? v.p[ro + dim_off(v.col, (uint32_t)(k + 1))] : 0.0, emax, d1);
#pragma unroll
            for (int p = 0; p < S; ++p)
                *reinterpret_cast<uint32_t *>(dst + p * plane + k) = bf16x2_of_digits(d0[p], d1[p]);
        }
    }
}

// The same for views whose k index runs in contiguous, 16-byte aligned groups of G
// (2 or 4) doubles: a lane loads a group with G/2 16-byte loads and stores G
// BF16 digits per plane in one 4- or 8-byte store.  Same digits and scales as
// split_rows_kernel.
__device__ __forceinline__ uint32_t abshi(double x) {  // high word of |x|: orders |x| by exponent
    return (uint32_t)__double2hiint(x) & 0x7FFFFFFFu;
}

template <int G>
__device__ __forceinline__ void load_group(const double *p, double (&x)[G]) {
#pragma unroll
    for (int h = 0; h < G / 2; ++h) {
        const double2 t = __ldg(reinterpret_cast<const double2 *>(p) + h);
        x[2 * h] = t.x;
        x[2 * h + 1] = t.y;
    }
}

// the S digit planes of one group of G values, stored at dst + p * plane
template <int S, int G>
__device__ __forceinline__ void store_group_digits(const double (&x)[G], int emax, __nv_bfloat16 *dst, size_t plane) {
    float d[G][S];
#pragma unroll
    for (int g = 0; g < G; ++g) split_digits<S>(x[g], emax, d[g]);
#pragma unroll
    for (int p = 0; p < S; ++p) {
        const uint32_t lo = bf16x2_of_digits(d[0][p], d[1][p]);
        if constexpr (G == 4) {
            *reinterpret_cast<uint2 *>(dst + p * plane) = make_uint2(lo, bf16x2_of_digits(d[2][p], d[3][p]));
        } else {
            *reinterpret_cast<uint32_t *>(dst + p * plane) = lo;
        }
    }
}

// Short rows (K * 8 bytes within L2 for the whole grid): a warp per row, the second
// pass re-reads the row from L2; UNR groups per lane in flight in the first.
template <int S, int G>
__global__ void __launch_bounds__(256) split_rows_vec_kernel(int rows, int K, int kpad, MatView v,
                                                             __nv_bfloat16 *__restrict__ planes, size_t plane,
                                                             double *__restrict__ scale) {
    constexpr int UNR = G == 4 ? 2 : 4, step = 32 * G;
    const int lane = threadIdx.x & 31;
    const int warp = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
    const int nwarps = (int)(((size_t)gridDim.x * blockDim.x) >> 5);
    for (int r = warp; r < rows; r += nwarps) {
        const double *row = v.p + dim_off(v.row, (uint32_t)r);
        uint32_t m = 0;  // maximum of the high words of |x|: the row's exponent
        int k = G * lane;
        for (; k + (UNR - 1) * step < K; k += UNR * step) {
            double x[UNR][G];
#pragma unroll
            for (int u = 0; u < UNR; ++u) load_group<G>(row + dim_off(v.col, (uint32_t)(k + u * step)), x[u]);
#pragma unroll
            for (int u = 0; u < UNR; ++u)
#pragma unroll
                for (int g = 0; g < G; ++g) m = max(m, abshi(x[u][g]));
        }
        for (; k < K; k += step) {
            double x[G];
            load_group<G>(row + dim_off(v.col, (uint32_t)k), x);
#pragma unroll
            for (int g = 0; g < G; ++g) m = max(m, abshi(x[g]));
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, off));
        const int emax = (int)((m >> 20) & 0x7FF);  // 0: zero (or denormal) row
        if (lane == 0) scale[r] = emax ? __longlong_as_double((long long)(emax + 1) << 52) : 1.0;
        __nv_bfloat16 *dst = planes + (size_t)r * kpad;
        for (k = G * lane; k < kpad; k += step) {
            double x[G];
            if (k < K) {
                load_group<G>(row + dim_off(v.col, (uint32_t)k), x);
            } else {
#pragma unroll
                for (int g = 0; g < G; ++g) x[g] = 0.0;
            }
            store_group_digits<S, G>(x, emax, dst + k, plane);
        }
    }
}

// Pass 2 for long rows in 16-byte groups, after rowmax_kernel: a block takes 256 G
// consecutive k of one row (one group per thread) and writes their digits; no shared
// memory and no exchange, so the loads and stores stream.
template <int S, int G>
__global__ void __launch_bounds__(256) split_planes_vec_kernel(int rows, int K, int kpad, MatView v,
                                                               const unsigned long long *__restrict__ rmax,
                                                               __nv_bfloat16 *__restrict__ planes, size_t plane,
                                                               double *__restrict__ scale) {
    constexpr int chunk = 256 * G;
    const int nch = (kpad + chunk - 1) / chunk;
    const long long units = (long long)rows * nch;
    for (long long u = blockIdx.x; u < units; u += gridDim.x) {
        const int r = (int)(u / nch), c = (int)(u - (long long)r * nch);
        const int emax = (int)((rmax[r] >> 20) & 0x7FF);  // 0: zero (or denormal) row
        if (c == 0 && threadIdx.x == 0) scale[r] = emax ? __longlong_as_double((long long)(emax + 1) << 52) : 1.0;
        const int k = c * chunk + G * threadIdx.x;
        if (k >= kpad) continue;
        double x[G];
        if (k < K) {
            load_group<G>(v.p + dim_off(v.row, (uint32_t)r) + dim_off(v.col, (uint32_t)k), x);
        } else {
#pragma unroll
            for (int g = 0; g < G; ++g) x[g] = 0.0;
        }
        store_group_digits<S, G>(x, emax, planes + (size_t)r * kpad + k, plane);
    }
}

// Rows of up to kSmemRowK doubles: a block per row stages the row in shared memory
// on its one read from HBM (UNR groups per thread in flight), takes the maximum, and
// writes the digits from shared memory.
constexpr int kSmemRowK = 8192;
template <int S, int G>
__global__ void __launch_bounds__(256) split_rows_smem_kernel(int rows, int K, int kpad, MatView v,
                                                              __nv_bfloat16 *__restrict__ planes, size_t plane,
                                                              double *__restrict__ scale) {
    constexpr int UNR = 4, step = 256 * G;
    extern __shared__ double2 srow[];  // K doubles
    __shared__ uint32_t red[8];
    const int tid = threadIdx.x, lane = tid & 31;
    for (int r = blockIdx.x; r < rows; r += gridDim.x) {
        const double *row = v.p + dim_off(v.row, (uint32_t)r);
        uint32_t m = 0;  // maximum of the high words of |x|
        int k = G * tid;
        for (; k + (UNR - 1) * step < K; k += UNR * step) {
            double x[UNR][G];
#pragma unroll
            for (int u = 0; u < UNR; ++u) load_group<G>(row + dim_off(v.col, (uint32_t)(k + u * step)), x[u]);
#pragma unroll
            for (int u = 0; u < UNR; ++u) {
#pragma unroll
                for (int h = 0; h < G / 2; ++h)
                    srow[(k + u * step) / 2 + h] = make_double2(x[u][2 * h], x[u][2 * h + 1]);
#pragma unroll
                for (int g = 0; g < G; ++g) m = max(m, abshi(x[u][g]));
            }
        }
        for (; k < K; k += step) {
            double x[G];
            load_group<G>(row + dim_off(v.col, (uint32_t)k), x);
#pragma unroll
            for (int h = 0; h < G / 2; ++h) srow[k / 2 + h] = make_double2(x[2 * h], x[2 * h + 1]);
#pragma unroll
            for (int g = 0; g < G; ++g) m = max(m, abshi(x[g]));
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, off));
        if (lane == 0) red[tid >> 5] = m;
        __syncthreads();  // the row and the warp maxima are in shared memory
#pragma unroll
        for (int q = 0; q < 8; ++q) m = max(m, red[q]);
        const int emax = (int)((m >> 20) & 0x7FF);  // 0: zero (or denormal) row
        if (tid == 0) scale[r] = emax ? __longlong_as_double((long long)(emax + 1) << 52) : 1.0;
        __nv_bfloat16 *dst = planes + (size_t)r * kpad;
        for (k = G * tid; k < kpad; k += step) {
            double x[G];
#pragma unroll
            for (int h = 0; h < G / 2; ++h) {
                const double2 t = k < K ? srow[k / 2 + h] : make_double2(0.0, 0.0);
                x[2 * h] = t.x;
                x[2 * h + 1] = t.y;
            }
            store_group_digits<S, G>(x, emax, dst + k, plane);
        }
        __syncthreads();  // srow and red are rewritten for the next row
    }
}

template <int S, bool ROWC>
__global__ void split_planes_kernel(int rows, int rows_pad, int K, int kpad, int nkt, MatView v,
                                    const unsigned long long *rmax, __nv_bfloat16 *planes, double *scale) {
    planes_block<S, ROWC>(rows, rows_pad, K, kpad, kpad, (size_t)rows_pad * kpad, v, rmax, planes, scale,
                          (int)(blockIdx.x / nkt) * 32, (int)(blockIdx.x % nkt) * 32);
}

// Grouped forms (batched solve): blockIdx.y = part; each part's rows go to
// packed rows row0.. of the shared planes (row pitch = the packed kpad).
template <bool ROWC>
__global__ void grouped_rowmax_kernel(const GroupedSplitOperandPart *parts, const int *active,
                                      unsigned long long *rmax) {
    const GroupedSplitOperandPart &P = parts[blockIdx.y];
    if (!active[P.sys]) return;
    const int nkg = (P.K + 32 * kRowmaxKT - 1) / (32 * kRowmaxKT);
    const int nblocks = (P.rows + 31) / 32 * nkg;
    for (int b = blockIdx.x; b < nblocks; b += gridDim.x)
        rowmax_block<ROWC>(P.rows, P.K, P.v, rmax + P.row0, (b / nkg) * 32, (b % nkg) * 32 * kRowmaxKT);
}

template <int S, bool ROWC>
__global__ void grouped_planes_kernel(const GroupedSplitOperandPart *parts, const int *active, int total_rows,
                                      int pitch, const unsigned long long *rmax, __nv_bfloat16 *planes,
                                      double *scale) {
    const GroupedSplitOperandPart &P = parts[blockIdx.y];
    if (!active[P.sys]) return;
    const int rows_pad = (P.rows + BM - 1) / BM * BM, kpad = (P.K + BK - 1) / BK * BK;
    const int nkt = kpad / 32, nblocks = rows_pad / 32 * nkt;
    for (int b = blockIdx.x; b < nblocks; b += gridDim.x)
        planes_block<S, ROWC>(P.rows, rows_pad, P.K, kpad, pitch, (size_t)total_rows * pitch, P.v, rmax + P.row0,
                              planes + (size_t)P.row0 * pitch, scale + P.row0, (b / nkt) * 32, (b % nkt) * 32);
}

__global__ void splitk_reduce(int M, int N, int splits, double alpha, const double *ws, double beta,
                              OutView C) {
    const size_t total = (size_t)M * N;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < total;
         idx += (size_t)gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int z = 0; z < splits; ++z) s += ws[z * total + idx];
        const int m = (int)(idx / N), n = (int)(idx % N);
        double *cp = C.p + dim_off(C.row, (uint32_t)m) + dim_off(C.col, (uint32_t)n);
        double out = alpha * s;
        if (beta != 0.0) out = fma(beta, *cp, out);
        *cp = out;
    }
}

PFN_cuTensorMapEncodeTiled_v12000 get_encode() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        CCSD_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q));
        if (q != cudaDriverEntryPointSuccess || !p) throw Error(-2, "cuTensorMapEncodeTiled unavailable");
        fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    }
    return fn;
}

void encode_raw(CUtensorMap *map, void *planes, int kpad, int nslices, int rows, int box_rows) {
    cuuint64_t gdim[2] = {(cuuint64_t)kpad, (cuuint64_t)nslices * rows};
    cuuint64_t gstride[1] = {(cuuint64_t)kpad * 2};
    cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)box_rows};
    cuuint32_t estride[2] = {1, 1};
    CUresult r = get_encode()(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, planes, gdim, gstride, box, estride,
                              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) throw Error(-2, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
}

void encode(CUtensorMap *map, const SplitOperand &op, int box_rows) {
    encode_raw(map, op.planes, op.kpad, op.nslices, op.rows_pad, box_rows);
}

template <int S, int BN, int NSTF, int MINB>
constexpr size_t kernel_smem() {
    constexpr int NST = NSTF > 0 ? NSTF : num_stages(S, BN);
    // two-per-SM variants request at least 80 KB so that no third CTA (and its
    // TMEM allocation) can become resident on the SM
    constexpr size_t need = (size_t)NST * stage_bytes(S, BN) + epi_offset() + epi_bytes(BN) + 1024;
    return (MINB > 1 && need < 80 * 1024) ? 80 * 1024 : need;
}

template <int S, int BN, int NSTF, int MINB, class Jobs>
void set_smem_attr() {
    static bool attr = false;
    if (!attr) {
        CCSD_CUDA(cudaFuncSetAttribute(split_gemm_kernel<S, BN, NSTF, MINB, Jobs>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)kernel_smem<S, BN, NSTF, MINB>()));
        attr = true;
    }
}

// Whether every column offset dim_off(C.col, n), n < N, lies in [0, 2^31): the strides
// are non-negative and the largest offset, at the last index of each level, fits.
bool col_offsets_32(const OutView &C, int N) {
    const Dim &d = C.col;
    if (N <= 0) return true;
    if (d.s0 < 0 || d.s1 < 0 || d.s2 < 0) return false;
    int64_t e2 = d.e2 == 0xFFFFFFFFu ? N : std::min<int64_t>(d.e2, N);
    int64_t q = d.e2 == 0xFFFFFFFFu ? 1 : ((int64_t)N + d.e2 - 1) / d.e2;  // extent of the upper levels
    int64_t mx = (e2 - 1) * d.s2;
    if (d.e2 != 0xFFFFFFFFu) {
        if (d.e1 == 0xFFFFFFFFu) {
            mx += (q - 1) * d.s1;
        } else {
            mx += (std::min<int64_t>(d.e1, q) - 1) * d.s1 + ((q + d.e1 - 1) / d.e1 - 1) * d.s0;
        }
    }
    return mx < (1LL << 31);
}

int num_sms();

template <int S, int BN, int NSTF = 0, int MINB = 1>
void launch_t(const SplitOperand &A, const SplitOperand &B, int M, int N, double alpha, double beta,
              const OutView &C, double *ws, size_t ws_elems, int *d_err, cudaStream_t st) {
    constexpr size_t smem = kernel_smem<S, BN, NSTF, MINB>();
    static_assert(MINB * smem <= 227 * 1024 && MINB * tmem_cols(BN) <= 512, "co-resident CTAs must fit");
    set_smem_attr<S, BN, NSTF, MINB, SingleJobs>();
    alignas(64) CUtensorMap ta, tb;
    encode(&ta, A, BM);
    encode(&tb, B, BN);
    const int nkb = A.kpad / BK;
    const int tiles_m = (M + BM - 1) / BM, tiles_n = (N + BN - 1) / BN;
    const long tiles = (long)tiles_m * tiles_n;
    // split K for parallelism when the tiles are fewer than the CTA slots (SMs x MINB), and to
    // keep the int32 level-0 sums bounded.  From the fewest splits that fill every slot up to
    // twice that, the count with the fewest waves per unit of work is taken (the smallest of
    // equals): 114 tiles on 152 slots take 4 splits, three full waves, rather than 2, whose
    // second wave is half empty.
    int splits = 1;
    const long slots = (long)num_sms() * MINB;
    if (tiles < slots) {
        const long kcap = std::max(1, nkb / 8);
        const long s0 = std::min<long>((slots + tiles - 1) / tiles, kcap);
        long best_s = s0;
        double best = (double)((tiles * s0 + slots - 1) / slots) / (double)s0;
        for (long s = s0 + 1; s <= std::min<long>(2 * s0, kcap); ++s) {
            const double c = (double)((tiles * s + slots - 1) / slots) / (double)s;
            if (c < best - 1e-12) {
                best = c;
                best_s = s;
            }
        }
        splits = (int)best_s;
    }
    splits = std::max(splits, (nkb + kMaxKbPerSplit - 1) / kMaxKbPerSplit);
    while (splits > 1 && (size_t)splits * M * N > ws_elems) --splits;
    if ((nkb + splits - 1) / splits > kMaxKbPerSplit)
        throw Error(-7, "split GEMM: K too long for the available split-K workspace");
    int kbps = (nkb + splits - 1) / splits;
    splits = (nkb + kbps - 1) / kbps;
    dim3 grid((unsigned)(tiles_m * tiles_n), 1, splits);
    SingleJobs jobs;
    jobs.splits = splits;
    jobs.M = M;
    jobs.N = N;
    jobs.tiles_m = tiles_m;
    jobs.tiles_n = tiles_n;
    jobs.nkb_total = nkb;
    jobs.kb_per_split = kbps;
    jobs.scaleA = A.scale;
    jobs.scaleB = B.scale;
    jobs.alpha = alpha;
    jobs.beta = beta;
    jobs.C = C;
    jobs.ws = ws;
    split_gemm_kernel<S, BN, NSTF, MINB, SingleJobs><<<grid, kThreads, smem, st>>>(ta, tb, A.rows_pad, B.rows_pad,
                                                                                 jobs, d_err);
    CCSD_LAUNCH_CHECK();
    if (splits > 1) {
        const size_t total = (size_t)M * N;
        const int blocks = (int)std::min<size_t>((total + 255) / 256, 4096);
        splitk_reduce<<<blocks, 256, 0, st>>>(M, N, splits, alpha, ws, beta, C);
        CCSD_LAUNCH_CHECK();
    }
}

int num_sms() {
    static int n = 0;
    if (!n) {
        int dev = 0;
        CCSD_CUDA(cudaGetDevice(&dev));
        CCSD_CUDA(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev));
        if (n <= 0) n = 148;
    }
    return n;
}

// The persistent kernel: as many CTAs as fit (MINB per SM, at most one per work item).
template <int S, int BN, int NST, int MINB>
void launch_p(const SplitOperand &A, const SplitOperand &B, int M, int N, double alpha, double beta,
              const OutView &C, double *ws, size_t ws_elems, int *d_err, cudaStream_t st) {
    // eight epilogue warps where BN splits into two 32-column slices, else four; 16 C loads in
    // flight per thread with one CTA per SM, 8 with two (the register budget of two CTAs)
    constexpr int EW = BN % 64 == 0 ? 8 : 4, KCB = MINB == 1 ? 16 : 8;
    constexpr int BW = BN / (EW / 4);
    constexpr int threads = 64 + 32 * EW;
    constexpr size_t need = (size_t)NST * stage_bytes(S, BN) + pbars_bytes() + EW * epi_bytes(BW) + 1024;
    // two-per-SM variants request at least 80 KB so that no third CTA (and its TMEM) fits
    constexpr size_t smem = (MINB > 1 && need < 80 * 1024) ? 80 * 1024 : need;
    static_assert(MINB * smem <= 227 * 1024 && MINB * ptmem_cols(BN) <= 512, "co-resident CTAs must fit");
    static bool attr = false;
    if (!attr) {
        CCSD_CUDA(cudaFuncSetAttribute(split_gemm_persistent_kernel<S, BN, NST, MINB, EW, KCB>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        attr = true;
    }
    alignas(64) CUtensorMap ta, tb;
    encode(&ta, A, BM);
    encode(&tb, B, BN);
    const int nkb = A.kpad / BK;
    const int tiles_m = (M + BM - 1) / BM, tiles_n = (N + BN - 1) / BN;
    const long tiles = (long)tiles_m * tiles_n;
    const int slots = num_sms() * MINB;
    // split K when the tiles alone leave CTAs idle, and to keep the int32 level-0 sums bounded
    int splits = 1;
    if (tiles < slots) {
        splits = (int)std::min<long>((slots + tiles - 1) / tiles, std::max(1, nkb / 8));
    } else if (tiles < 4L * slots && nkb >= 256) {
        // long K over a few rounds of tiles: the split count (at most 8) that leaves the
        // last round fullest, the smaller on a tie
        double best = 0.0;
        for (int sp = 1; sp <= 8 && nkb / sp >= 32; ++sp) {
            if (sp > 1 && (size_t)sp * M * N > ws_elems) break;
            const long w = tiles * sp, rounds = (w + slots - 1) / slots;
            const double eff = (double)w / ((double)rounds * slots);
            if (eff > best + 0.02) {
                best = eff;
                splits = sp;
            }
        }
    }
    splits = std::max(splits, (nkb + kMaxKbPerSplit - 1) / kMaxKbPerSplit);
    while (splits > 1 && (size_t)splits * M * N > ws_elems) --splits;
    if ((nkb + splits - 1) / splits > kMaxKbPerSplit)
        throw Error(-7, "split GEMM: K too long for the available split-K workspace");
    int kbps = (nkb + splits - 1) / splits;
    splits = (nkb + kbps - 1) / kbps;
    const long nwork = tiles * splits;
    if (nwork >= (1L << 31)) throw Error(-7, "split GEMM: too many tiles");
    SingleJobs jobs;
    jobs.c32 = col_offsets_32(C, N);
    jobs.splits = splits;
    jobs.M = M;
    jobs.N = N;
    jobs.tiles_m = tiles_m;
    jobs.tiles_n = tiles_n;
    jobs.nkb_total = nkb;
    jobs.kb_per_split = kbps;
    jobs.scaleA = A.scale;
    jobs.scaleB = B.scale;
    jobs.alpha = alpha;
    jobs.beta = beta;
    jobs.C = C;
    jobs.ws = ws;
    const int grid = (int)std::min<long>(nwork, slots);
    split_gemm_persistent_kernel<S, BN, NST, MINB, EW, KCB><<<grid, threads, smem, st>>>(ta, tb, A.rows_pad, B.rows_pad,
                                                                               jobs, (int)nwork, d_err);
    CCSD_LAUNCH_CHECK();
    if (splits > 1) {
        const size_t total = (size_t)M * N;
        const int blocks = (int)std::min<size_t>((total + 255) / 256, 4096);
        splitk_reduce<<<blocks, 256, 0, st>>>(M, N, splits, alpha, ws, beta, C);
        CCSD_LAUNCH_CHECK();
    }
}

template <int S>
void launch_s(const SplitOperand &A, const SplitOperand &B, int M, int N, double alpha, double beta,
              const OutView &C, double *ws, size_t ws_elems, int *d_err, cudaStream_t st) {
    // the column tile with the fewest column tiles (passes over A: the pair-form
    // ladder's N = o(o-1)/2 = 276 runs 13% faster on two 160-wide tiles than on
    // three 96-wide ones), then the smallest padded width ceil(N / BN) * BN
    static const int cand[] = {160, 128, 96, 64, 32};
    int bn = 32;
    long best_t = -1, best_w = -1;
    for (int c : cand) {
        const long t = (N + c - 1) / c, w = t * c;
        if (best_t < 0 || t < best_t || (t == best_t && w < best_w)) {
            best_t = t;
            best_w = w;
            bn = c;
        }
    }
    // short K on a narrow tile: a few stages and two CTAs per SM, so one CTA's
    // pipeline fill and epilogue overlap the other's main loop
    const int nkb = A.kpad / BK;
    // K <= 128: the main loop is a few k-blocks and the epilogue's C traffic
    // dominates, so the narrow two-per-SM tiles win even for wide N
    if (nkb <= 4 && bn > 64) bn = 64;
    if (nkb <= 64 && bn <= 64) {
        constexpr int st32 = std::max(2, std::min(3, (100 * 1024) / stage_bytes(S, 32)));
        constexpr int st64 = std::max(2, std::min(3, (100 * 1024) / stage_bytes(S, 64)));
        if (bn == 32)
            launch_p<S, 32, st32, 2>(A, B, M, N, alpha, beta, C, ws, ws_elems, d_err, st);
        else
            launch_p<S, 64, st64, 2>(A, B, M, N, alpha, beta, C, ws, ws_elems, d_err, st);
        return;
    }
    // long K on at most two 160-wide column tiles (the pair-form ladder): a tile's fill and
    // epilogue are a small share of its main loop, and 160 columns (not a persistent width)
    // cut the passes over A; everything else runs persistent, at most 128 columns wide
    if (bn == 160 && nkb >= 512 && (N + 159) / 160 <= 2) {
        launch_t<S, 160>(A, B, M, N, alpha, beta, C, ws, ws_elems, d_err, st);
        return;
    }
    switch (bn) {
        case 160:
        case 128: launch_p<S, 128, num_stages(S, 128), 1>(A, B, M, N, alpha, beta, C, ws, ws_elems, d_err, st); break;
        case 96: launch_p<S, 96, num_stages(S, 96), 1>(A, B, M, N, alpha, beta, C, ws, ws_elems, d_err, st); break;
        case 64: launch_p<S, 64, num_stages(S, 64), 1>(A, B, M, N, alpha, beta, C, ws, ws_elems, d_err, st); break;
        default: launch_p<S, 32, num_stages(S, 32), 1>(A, B, M, N, alpha, beta, C, ws, ws_elems, d_err, st); break;
    }
}

template <int S, int BN>
void launch_grouped(const PackedSplit &A, const PackedSplit &B, const GroupedSplitPart *d_parts, int nparts,
                    int total_tiles, const int *active, int *d_err, cudaStream_t st) {
    constexpr size_t smem = kernel_smem<S, BN, 0, 1>();
    set_smem_attr<S, BN, 0, 1, GroupedJobs>();
    alignas(64) CUtensorMap ta, tb;
    encode_raw(&ta, A.planes, A.kpad, A.nslices, A.rows, BM);
    encode_raw(&tb, B.planes, B.kpad, B.nslices, B.rows, BN);
    GroupedJobs jobs;
    jobs.parts = d_parts;
    jobs.nparts = nparts;
    jobs.active = active;
    split_gemm_kernel<S, BN, 0, 1, GroupedJobs><<<total_tiles, kThreads, smem, st>>>(ta, tb, A.rows, B.rows, jobs,
                                                                                   d_err);
    CCSD_LAUNCH_CHECK();
}

}  // namespace

// ---------------------------------------------------------------------------
void packed_split_alloc(PackedSplit &op, int rows, int kpad, int nslices) {
    packed_split_free(op);
    const size_t bytes = (size_t)nslices * rows * kpad * 2;
    cudaError_t e = cudaMalloc(&op.planes, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        op.planes = nullptr;
        throw Error(-3, "packed split planes: cudaMalloc of " + std::to_string(bytes) + " bytes failed");
    }
    CCSD_CUDA(cudaMemset(op.planes, 0, bytes));
    CCSD_CUDA(cudaMalloc(&op.scale, sizeof(double) * rows));
    CCSD_CUDA(cudaMalloc(&op.rmax, sizeof(unsigned long long) * rows));
    op.rows = rows;
    op.kpad = kpad;
    op.nslices = nslices;
    op.bytes = bytes;
}

void packed_split_free(PackedSplit &op) {
    if (op.planes) cudaFree(op.planes);
    if (op.scale) cudaFree(op.scale);
    if (op.rmax) cudaFree(op.rmax);
    op = PackedSplit();
}

void grouped_split_operand_launch(PackedSplit &op, const GroupedSplitOperandPart *d_parts, int nparts,
                                  int max_rows, int max_kpad, bool rowc, const int *active, cudaStream_t st) {
    if (nparts <= 0) return;
    const dim3 thr(32, 8);
    CCSD_CUDA(cudaMemsetAsync(op.rmax, 0, sizeof(unsigned long long) * op.rows, st));
    const int nkg = (max_kpad + 32 * kRowmaxKT - 1) / (32 * kRowmaxKT);
    const int rblocks = std::max(1, std::min(1024, (max_rows + 31) / 32 * nkg));
    const int pblocks = std::max(1, std::min(4096, (max_rows + BM - 1) / BM * (BM / 32) * (max_kpad / 32)));
    if (rowc)
        grouped_rowmax_kernel<true><<<dim3(rblocks, nparts), thr, 0, st>>>(d_parts, active, op.rmax);
    else
        grouped_rowmax_kernel<false><<<dim3(rblocks, nparts), thr, 0, st>>>(d_parts, active, op.rmax);
    CCSD_LAUNCH_CHECK();
    __nv_bfloat16 *pl = (__nv_bfloat16 *)op.planes;
#define CCSD_GSPLIT_CASE(S_)                                                                                     \
    case S_:                                                                                                     \
        if (rowc)                                                                                                \
            grouped_planes_kernel<S_, true><<<dim3(pblocks, nparts), thr, 0, st>>>(d_parts, active, op.rows,    \
                                                                                   op.kpad, op.rmax, pl, op.scale); \
        else                                                                                                     \
            grouped_planes_kernel<S_, false><<<dim3(pblocks, nparts), thr, 0, st>>>(d_parts, active, op.rows,   \
                                                                                    op.kpad, op.rmax, pl, op.scale); \
        break;
    switch (op.nslices) {
        CCSD_GSPLIT_CASE(2)
        CCSD_GSPLIT_CASE(3)
        CCSD_GSPLIT_CASE(4)
        default: throw Error(-1, "nslices must be 2, 3 or 4");
    }
#undef CCSD_GSPLIT_CASE
    CCSD_LAUNCH_CHECK();
}

int grouped_split_bn(int max_n) { return max_n <= 64 ? 64 : 128; }

void grouped_split_gemm_launch(const PackedSplit &A, const PackedSplit &B, int bn, const GroupedSplitPart *d_parts,
                               int nparts, int total_tiles, const int *active, int *d_err, cudaStream_t st) {
    if (nparts <= 0 || total_tiles <= 0) return;
    if (A.kpad != B.kpad || A.nslices != B.nslices) throw Error(-1, "grouped split operands disagree");
    if (bn != 64 && bn != 128) throw Error(-1, "grouped split tile width must be 64 or 128");
#define CCSD_GGEMM_CASE(S_)                                                                                 \
    case S_:                                                                                                \
        if (bn == 64)                                                                                       \
            launch_grouped<S_, 64>(A, B, d_parts, nparts, total_tiles, active, d_err, st);                  \
        else                                                                                                \
            launch_grouped<S_, 128>(A, B, d_parts, nparts, total_tiles, active, d_err, st);                 \
        break;
    switch (A.nslices) {
        CCSD_GGEMM_CASE(2)
        CCSD_GGEMM_CASE(3)
        CCSD_GGEMM_CASE(4)
        default: throw Error(-1, "nslices must be 2, 3 or 4");
    }
#undef CCSD_GGEMM_CASE
}

// ---------------------------------------------------------------------------
// Whether k runs through the view in contiguous groups of G doubles that start on
// 16-byte boundaries: unit stride in k, G dividing K and the innermost extent of
// the k index, and every other stride (of k and of the row index) even.
static bool k_groups(const MatView &v, int K, int G) {
    const auto even = [](int64_t s) { return (s & 1) == 0; };
    if (v.col.s2 != 1 || K % G != 0 || ((uintptr_t)v.p & 15) != 0) return false;
    if (v.col.e2 != 0xFFFFFFFFu) {
        if (v.col.e2 % G != 0 || !even(v.col.s1)) return false;
        if (v.col.e1 != 0xFFFFFFFFu && !even(v.col.s0)) return false;
    }
    if (!even(v.row.s2)) return false;
    if (v.row.e2 != 0xFFFFFFFFu) {
        if (!even(v.row.s1)) return false;
        if (v.row.e1 != 0xFFFFFFFFu && !even(v.row.s0)) return false;
    }
    return true;
}

// A view of 16-byte groups (k_groups): rows up to kSmemRowK long are staged in shared
// memory, a block per row (one HBM read); short rows (under 1024, whose re-read stays
// in L2) take a warp per row; longer rows take two passes (row maxima, then the digits
// streamed).  Always returns true.
template <int S, int G>
static bool launch_split_vec_g(int rows, int K, int kpad, const MatView &v, __nv_bfloat16 *pl, size_t plane,
                               double *scale, unsigned long long *rmax, cudaStream_t st) {
    if (K < 1024) {
        const int grid = (int)std::min<long long>((rows + 7) / 8, 152LL * 8);
        split_rows_vec_kernel<S, G><<<grid, 256, 0, st>>>(rows, K, kpad, v, pl, plane, scale);
        CCSD_LAUNCH_CHECK();
        return true;
    }
    if (K > kSmemRowK) {  // two passes: row maxima, then the digits streamed in 16-byte groups
        const int nrt = (rows + 31) / 32;
        const long long nkg = (kpad + 32 * kRowmaxKT - 1) / (32 * kRowmaxKT);
        CCSD_CUDA(cudaMemsetAsync(rmax, 0, sizeof(unsigned long long) * rows, st));
        rowmax_kernel<false><<<(unsigned)(nrt * nkg), dim3(32, 8), 0, st>>>(rows, K, (int)nkg, v, rmax);
        CCSD_LAUNCH_CHECK();
        const long long units = (long long)rows * ((kpad + 256 * G - 1) / (256 * G));
        const int grid = (int)std::min<long long>(units, 152LL * 8 * 4);
        split_planes_vec_kernel<S, G><<<grid, 256, 0, st>>>(rows, K, kpad, v, rmax, pl, plane, scale);
        CCSD_LAUNCH_CHECK();
        return true;
    }
    const size_t smem = sizeof(double) * (size_t)K;
    static unsigned long long attr_set = 0;  // per device (the attribute is per context)
    int dev = 0;
    CCSD_CUDA(cudaGetDevice(&dev));
    if (dev < 64 && !(attr_set >> dev & 1ull)) {
        CCSD_CUDA(cudaFuncSetAttribute(split_rows_smem_kernel<S, G>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)(sizeof(double) * kSmemRowK)));
        attr_set |= 1ull << dev;
    }
    const long long per_sm = std::max<long long>(1, std::min<long long>(8, (200LL << 10) / (long long)(smem + 1024)));
    const int grid = (int)std::min<long long>(rows, 152LL * per_sm);
    split_rows_smem_kernel<S, G><<<grid, 256, smem, st>>>(rows, K, kpad, v, pl, plane, scale);
    CCSD_LAUNCH_CHECK();
    return true;
}

template <int S>
static bool launch_split_vec(int G, int rows, int K, int kpad, const MatView &v, __nv_bfloat16 *pl, size_t plane,
                             double *scale, unsigned long long *rmax, cudaStream_t st) {
    return G == 4 ? launch_split_vec_g<S, 4>(rows, K, kpad, v, pl, plane, scale, rmax, st)
                  : launch_split_vec_g<S, 2>(rows, K, kpad, v, pl, plane, scale, rmax, st);
}

void split_operand_kernel_launch(SplitOperand &op, int rows, int K, const MatView &v, cudaStream_t st) {
    const int nkt = op.kpad / 32, nrt = op.rows_pad / 32;
    const long long blocks = (long long)nkt * nrt;
    if (blocks >= (1ll << 31)) throw Error(-7, "split operand too large");
    const dim3 thr(32, 8);
    // read along rows when the row index is the contiguous one
    const bool rowc = v.row.s2 == 1 && v.col.s2 != 1;
    __nv_bfloat16 *pl0 = (__nv_bfloat16 *)op.planes;
    const size_t plane0 = (size_t)op.rows_pad * op.kpad;
    const int G = rowc ? 0 : (k_groups(v, K, 4) ? 4 : (k_groups(v, K, 2) ? 2 : 0));
    if (G) {  // one HBM pass, 16-byte loads
        bool done = false;
        switch (op.nslices) {
            case 2: done = launch_split_vec<2>(G, rows, K, op.kpad, v, pl0, plane0, op.scale, op.rmax, st); break;
            case 3: done = launch_split_vec<3>(G, rows, K, op.kpad, v, pl0, plane0, op.scale, op.rmax, st); break;
            case 4: done = launch_split_vec<4>(G, rows, K, op.kpad, v, pl0, plane0, op.scale, op.rmax, st); break;
            default: throw Error(-1, "nslices must be 2, 3 or 4");
        }
        if (done) return;
    }
    if (!rowc && K <= 32768 && rows >= 8 * 152) {  // one pass, a warp per row
        const size_t plane = (size_t)op.rows_pad * op.kpad;
        const int grid = (int)std::min<long long>((rows + 7) / 8, 152LL * 8);
        switch (op.nslices) {
            case 2: split_rows_kernel<2><<<grid, 256, 0, st>>>(rows, K, op.kpad, v, pl0, plane, op.scale); break;
            case 3: split_rows_kernel<3><<<grid, 256, 0, st>>>(rows, K, op.kpad, v, pl0, plane, op.scale); break;
            case 4: split_rows_kernel<4><<<grid, 256, 0, st>>>(rows, K, op.kpad, v, pl0, plane, op.scale); break;
            default: throw Error(-1, "nslices must be 2, 3 or 4");
        }
        CCSD_LAUNCH_CHECK();
        return;
    }
    const long long nkg = (op.kpad + 32 * kRowmaxKT - 1) / (32 * kRowmaxKT);
    CCSD_CUDA(cudaMemsetAsync(op.rmax, 0, sizeof(unsigned long long) * op.rows_pad, st));
    __nv_bfloat16 *pl = (__nv_bfloat16 *)op.planes;
    if (rowc)
        rowmax_kernel<true><<<(unsigned)(nrt * nkg), thr, 0, st>>>(rows, K, nkg, v, op.rmax);
    else
        rowmax_kernel<false><<<(unsigned)(nrt * nkg), thr, 0, st>>>(rows, K, nkg, v, op.rmax);
    CCSD_LAUNCH_CHECK();
#define CCSD_SPLIT_CASE(S_)                                                                                  \
    case S_:                                                                                                  \
        if (rowc)                                                                                             \
            split_planes_kernel<S_, true><<<(unsigned)blocks, thr, 0, st>>>(rows, op.rows_pad, K, op.kpad, nkt, v, \
                                                                            op.rmax, pl, op.scale);           \
        else                                                                                                  \
            split_planes_kernel<S_, false><<<(unsigned)blocks, thr, 0, st>>>(rows, op.rows_pad, K, op.kpad, nkt, \
                                                                             v, op.rmax, pl, op.scale);      \
        break;
    switch (op.nslices) {
        CCSD_SPLIT_CASE(2)
        CCSD_SPLIT_CASE(3)
        CCSD_SPLIT_CASE(4)
        default: throw Error(-1, "nslices must be 2, 3 or 4");
    }
#undef CCSD_SPLIT_CASE
    CCSD_LAUNCH_CHECK();
}

void split_gemm_launch(const SplitOperand &A, const SplitOperand &B, int M, int N, double alpha, double beta,
                       const OutView &C, double *ws, size_t ws_elems, int *d_err, cudaStream_t st) {
    if (A.kpad != B.kpad || A.nslices != B.nslices) throw Error(-1, "split operands disagree");
    switch (A.nslices) {
        case 2: launch_s<2>(A, B, M, N, alpha, beta, C, ws, ws_elems, d_err, st); break;
        case 3: launch_s<3>(A, B, M, N, alpha, beta, C, ws, ws_elems, d_err, st); break;
        case 4: launch_s<4>(A, B, M, N, alpha, beta, C, ws, ws_elems, d_err, st); break;
        default: throw Error(-1, "nslices must be 2, 3 or 4");
    }
}

// One contraction on freshly split operands (the ccsd_gemm entry point).
void split_gemm_oneshot(int nslices, int M, int N, int K, double alpha, const MatView &A, const MatView &B,
                        double beta, const OutView &C, cudaStream_t st) {
    SplitEngine eng(nslices, st);
    eng.gemm(M, N, K, alpha, A, B, beta, C, 0, 0);
    const int err = eng.error_status();
    if (err) throw Error(-6, "split GEMM: a bounded device wait gave up (error word " + std::to_string(err) + ")");
}

// ---------------------------------------------------------------------------
SplitEngine::SplitEngine(int nslices, cudaStream_t st) : nslices_(nslices), st_(st) {
    if (nslices < 2 || nslices > 4) throw Error(-1, "nslices must be 2, 3 or 4");
    int dev = 0, major = 0, minor = 0;
    CCSD_CUDA(cudaGetDevice(&dev));
    CCSD_CUDA(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev));
    CCSD_CUDA(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev));
    if (major != 10 || minor != 3)
        throw Error(-7, "split-precision engine needs an sm_103 GPU (tcgen05); found sm_" +
                            std::to_string(major) + std::to_string(minor));
    CCSD_CUDA(cudaMalloc(&d_err_, sizeof(int)));
    CCSD_CUDA(cudaMemsetAsync(d_err_, 0, sizeof(int), st_));
    ws_elems_ = 32u << 20;  // split-K partials (256 MB)
    CCSD_CUDA(cudaMalloc(&ws_, ws_elems_ * sizeof(double)));
}

SplitEngine::~SplitEngine() {
    for (auto &kv : cache_) free_op(*kv.second);
    for (auto &kv : dyn_) free_op(*kv.second);
    free_op(scratch_[0]);
    free_op(scratch_[1]);
    if (d_err_) cudaFree(d_err_);
    if (ws_) cudaFree(ws_);
}

void SplitEngine::free_op(SplitOperand &op) {
    if (op.planes) cudaFree(op.planes);
    if (op.scale) cudaFree(op.scale);
    if (op.rmax) cudaFree(op.rmax);
    op.planes = nullptr;
    op.scale = nullptr;
    op.rmax = nullptr;
    op.bytes = 0;
}

// Rows are padded to a multiple of 32 for the splitter's tiles, not to the MMA
// tile: TMA boxes that run past an operand's rows read the next plane (or the
// map's zero fill after the last one), and those rows only reach output rows or
// columns the epilogue discards.  The planes together keep at least 160 rows so
// that no box (128 rows for A, at most 160 for B) is taller than the map.
static int split_rows_pad(int rows, int nslices) {
    const int r32 = (rows + 31) / 32 * 32;
    const int min_rows = ((160 + nslices - 1) / nslices + 31) / 32 * 32;
    return r32 > min_rows ? r32 : min_rows;
}

void SplitEngine::ensure(SplitOperand &op, int rows, int K) {
    const int rows_pad = split_rows_pad(rows, nslices_);
    const int kpad = (K + BK - 1) / BK * BK;
    const size_t need = (size_t)nslices_ * rows_pad * kpad * 2;
    if (!op.planes || need > op.bytes || (size_t)rows_pad > op.scale_cap) {
        // grow both to the largest seen, so that a scratch operand shared by a tall
        // thin and a square contraction settles after one update instead of being
        // re-allocated (a device synchronisation) on every one
        const size_t bytes = need > op.bytes ? need : op.bytes;
        const size_t cap = (size_t)rows_pad > op.scale_cap ? (size_t)rows_pad : op.scale_cap;
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(st_, &cs) != cudaSuccess) {
            cudaGetLastError();
            cs = cudaStreamCaptureStatusActive;  // the legacy stream while another one captures
        }
        if (cs != cudaStreamCaptureStatusNone)
            throw CaptureMiss("split planes: " + std::to_string(bytes) + " bytes wanted during graph capture");
        free_op(op);
        void *p = nullptr;
        cudaError_t e = cudaMalloc(&p, bytes);
        if (e != cudaSuccess) {
            cudaGetLastError();
            throw Error(-3, "split planes: cudaMalloc of " + std::to_string(bytes) + " bytes failed");
        }
        op.planes = p;
        op.bytes = bytes;
        CCSD_CUDA(cudaMalloc(&op.scale, sizeof(double) * cap));
        CCSD_CUDA(cudaMalloc(&op.rmax, sizeof(unsigned long long) * cap));
        op.scale_cap = cap;
    }
    op.rows = rows;
    op.rows_pad = rows_pad;
    op.K = K;
    op.kpad = kpad;
    op.nslices = nslices_;
}

void SplitEngine::split_into(SplitOperand &op, int rows, int K, const MatView &v) {
    ensure(op, rows, K);
    split_operand_kernel_launch(op, rows, K, v, st_);
}

SplitOperand *SplitEngine::operand(int key, int rows, int K, const MatView &v, int slot) {
    if (key == 0) {
        split_into(scratch_[slot], rows, K, v);
        return &scratch_[slot];
    }
    if (key < 0) {
        std::unique_ptr<SplitOperand> &op = dyn_[key];
        if (!op) op.reset(new SplitOperand());
        if (!dyn_valid_[key] || op->rows != rows || op->K != K) {
            split_into(*op, rows, K, v);
            dyn_valid_[key] = true;
        }
        return op.get();
    }
    auto it = cache_.find(key);
    if (it != cache_.end()) {
        SplitOperand *op = it->second.get();
        if (op->rows == rows && op->K == K) return op;
        free_op(*op);
        cache_.erase(it);
    }
    std::unique_ptr<SplitOperand> op(new SplitOperand());
    split_into(*op, rows, K, v);
    SplitOperand *raw = op.get();
    cache_[key] = std::move(op);
    return raw;
}

void SplitEngine::gemm(int M, int N, int K, double alpha, const MatView &A, const MatView &B, double beta,
                       const OutView &C, int cache_a, int cache_b) {
    if (prefer_swap(M, N, C)) {  // C^T = B A^T: long side / unit-stride output index in the rows
        gemm(N, M, K, alpha, B, A, beta, OutView{C.p, C.col, C.row}, cache_b, cache_a);
        return;
    }
    SplitOperand *a = operand(cache_a, M, K, A, 0);
    SplitOperand *b = operand(cache_b, N, K, B, 1);
    split_gemm_launch(*a, *b, M, N, alpha, beta, C, ws_, ws_elems_, d_err_, st_);
}

void SplitEngine::run(const SplitOperand &a, const SplitOperand &b, int M, int N, double alpha, double beta,
                      const OutView &C) {
    split_gemm_launch(a, b, M, N, alpha, beta, C, ws_, ws_elems_, d_err_, st_);
}

void SplitEngine::clear_error() { CCSD_CUDA(cudaMemsetAsync(d_err_, 0, sizeof(int), st_)); }

int SplitEngine::error_status() {
    int h = 0;
    CCSD_CUDA(cudaMemcpyAsync(&h, d_err_, sizeof(int), cudaMemcpyDeviceToHost, st_));
    CCSD_CUDA(cudaStreamSynchronize(st_));
    return h;
}

size_t SplitEngine::cached_bytes() const {
    size_t s = 0;
    for (auto &kv : cache_) s += kv.second->bytes;
    return s;
}

}  // namespace ccsd

namespace ccsd {
void set_last_error(const std::string &msg);
}

extern "C" int ccsd_debug_stall_split_mma(uint64_t stall_ns) {
    const unsigned long long v = stall_ns;
    const cudaError_t e = cudaMemcpyToSymbol(ccsd::g_stall_mma_ns, &v, sizeof v);
    if (e != cudaSuccess) {
        cudaGetLastError();
        ccsd::set_last_error(std::string("ccsd_debug_stall_split_mma: ") + cudaGetErrorString(e));
        return e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver ? CCSD_ERR_NO_DEVICE : CCSD_ERR_CUDA;
    }
    return CCSD_OK;
}
