// Grouped kernels of the batched solve: one launch applies the same operation
// of the amplitude update to every system of a batch (uneven nocc/nvir).
//
// Each descriptor array has one entry ("part") per system, in system order;
// every kernel first reads active[part.sys] and skips systems that have
// stopped iterating, so one captured CUDA graph serves every update of the
// batch while systems converge at different iterations.
#pragma once

#include <vector>

#include "common.h"

namespace ccsd {

// One system's share of a grouped contraction C = alpha A B^T + beta C.
struct GGemm {
    MatView A, B;
    OutView C;
    double alpha = 0.0, beta = 0.0;
    int M = 0, N = 0, K = 0, sys = 0;
    int splits = 1, kchunk = 0;  // split-K plan
    int tiles_m = 0, tiles_n = 0;
    int item_begin = 0;          // first work item of this part
    long long ws_off = 0;        // partial sums at ws + ws_off when splits > 1
};

struct GAxpby {  // Y = alpha X + beta Y over an R x C view grid
    MatView X;
    OutView Y;
    double alpha = 0.0, beta = 0.0;
    int R = 0, C = 0, sys = 0;
};

struct GAmp {  // tau / theta: (t1, t2) -> out1 (, out2)
    const double *t1 = nullptr, *t2 = nullptr;
    double *out1 = nullptr, *out2 = nullptr;
    int o = 0, v = 0, sys = 0;
};

struct GUpdate {  // t_new = numerator / D and |t_new - t_old|^2 partial sums
    const double *R = nullptr, *Rp = nullptr, *R1 = nullptr, *eo = nullptr, *ev = nullptr;
    const double *t1_old = nullptr, *t2_old = nullptr;
    double *t1_new = nullptr, *t2_new = nullptr;
    int o = 0, v = 0, sys = 0;
};

struct GDot {  // sum x . y
    const double *x = nullptr, *y = nullptr;
    long long n = 0;
    int sys = 0;
};

// Tile shapes of the grouped FP64 contraction (16 x 16 threads, TM x TN
// register micro-tile, BK = 16).
enum GTile { kTile64x64 = 0, kTile32x64, kTile64x32, kTile32x32, kTile128x64, kNumGTiles };
int gtile_bm(int cfg);
int gtile_bn(int cfg);

// A plan of one grouped contraction: tile shape and split-K target.
struct GGemmPlan {
    int cfg = kTile64x64;
    int target = 0;        // minimum work items wanted (split-K fills up to it)
    bool gemv = false;     // every part has M == 1 or N == 1
    bool akc = false, bkc = false;
    int total_items = 0;
    int grid = 0;
    size_t ws_elems = 0;
    bool any_split = false;
};

// Fill the split-K fields of `parts` for tile shape `cfg` and work-item target
// `target`, and return the launch plan.
GGemmPlan plan_grouped_gemm(std::vector<GGemm> &parts, int cfg, int target, int num_sms);

void launch_grouped_gemm(const GGemmPlan &plan, const GGemm *d_parts, int nparts, const int *active,
                         double *ws, cudaStream_t st);
void launch_grouped_axpby(const GAxpby *d_parts, int nparts, size_t max_elems, const int *active,
                          cudaStream_t st);
void launch_grouped_tau(const GAmp *d_parts, int nparts, size_t max_elems, const int *active, cudaStream_t st);
void launch_grouped_theta(const GAmp *d_parts, int nparts, size_t max_elems, const int *active,
                          cudaStream_t st);
// pair-form ladder: tau (t1) -> tau+ (out1), tau- (out2); R (out1) += unpack(S+ (t1), S- (t2))
void launch_grouped_tau_sym(const GAmp *d_parts, int nparts, size_t max_elems, const int *active,
                            cudaStream_t st);
void launch_grouped_unpack(const GAmp *d_parts, int nparts, size_t max_elems, const int *active,
                           cudaStream_t st);
// partials: nparts x grouped_partials_per_part(); part p's |dT|^2 pieces at p * per.
int grouped_partials_per_part();
void launch_grouped_update(const GUpdate *d_parts, int nparts, const int *active, double *partials,
                           cudaStream_t st);
void launch_grouped_dot(const GDot *d_parts, int nparts, const int *active, double *partials, cudaStream_t st);
// out[p] = sum of partials[p * per .. p * per + per) for active parts (fixed order).
void launch_grouped_sum(int nparts, const int *active, const double *partials, double *out, cudaStream_t st);

}  // namespace ccsd
