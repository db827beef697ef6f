// Split-precision contraction engine on the sm_103a tensor cores.
//
// An FP64 operand row x is written as
//     x = s * 2^-7 * (P0 + P1 + ... + P_{S-1}),  s = 2^ceil(log2 max|row|),
// where P0 = rint(x/s * 2^7) is an integer in [-128, 128] and every further
// plane carries the next 8 bits of the remainder, pre-scaled by 2^-8 per
// plane.  Every plane is exact in BF16.  tcgen05.mma (kind::f16, BF16 in,
// FP32 accumulate in TMEM) forms the plane products with level p+q < S:
//   * level 0 (P0 x P0) accumulates integers below 2^24 over K chunks of 1024
//     -- exact in FP32 -- and is drained into 32-bit integer registers;
//   * the higher levels share one FP32 accumulator (their rounding error is
//     already 2^-8 smaller).
// The epilogue forms C = alpha * sA * sB * 2^-14 * (I0 + F) + beta * C in FP64.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <memory>

#include "common.h"

namespace ccsd {

// Split form of a rows x K operand: S planes of [rows_pad][kpad] BF16
// (K-major, plane p at row offset p * rows_pad) plus one FP64 scale per row.
struct SplitOperand {
    void *planes = nullptr;  // __nv_bfloat16*
    double *scale = nullptr;
    unsigned long long *rmax = nullptr;  // row maxima (bit patterns) while splitting
    int rows = 0, rows_pad = 0, K = 0, kpad = 0, nslices = 0;
    size_t bytes = 0, scale_cap = 0;
};

class SplitEngine {
  public:
    SplitEngine(int nslices, cudaStream_t st);
    ~SplitEngine();
    void set_stream(cudaStream_t st) { st_ = st; }
    int nslices() const { return nslices_; }
    // C(m,n) = alpha * sum_k A(m,k) B(n,k) + beta C(m,n) on the tensor cores.
    // A nonzero cache key marks an operand view over constant data whose
    // split form is kept (keyed) between calls.
    void gemm(int M, int N, int K, double alpha, const MatView &A, const MatView &B, double beta,
              const OutView &C, int cache_a, int cache_b);
    // The two halves of gemm(): split (or fetch from the cache) one operand,
    // then run the tensor-core kernel on two prepared operands.
    SplitOperand *prepare(int key, int rows, int K, const MatView &v, int slot) {
        return operand(key, rows, K, v, slot);
    }
    void run(const SplitOperand &a, const SplitOperand &b, int M, int N, double alpha, double beta,
             const OutView &C);
    // The tensor-core tile is 128 rows by at most 128 columns: a product whose
    // row count is short and column count long runs faster transposed.
    static bool prefer_swap(int M, int N) { return M < 128 && N > M; }
    // also put the index of C with the smaller innermost stride in the rows
    // (TMEM lanes), so that the epilogue's lanes write the fewest sectors per
    // store; N >= 128 keeps the swapped problem's row dimension a full MMA tile
    static bool prefer_swap(int M, int N, const OutView &C) {
        const int64_t rs = C.row.s2 < 0 ? -C.row.s2 : C.row.s2;
        const int64_t cs = C.col.s2 < 0 ? -C.col.s2 : C.col.s2;
        return prefer_swap(M, N) || (cs < rs && N >= 128);
    }
    // Negative cache keys name amplitude-derived operands that several
    // contractions of one update share; begin_update() invalidates them.
    void begin_update() {
        for (auto &kv : dyn_valid_) kv.second = false;
    }
    // Device error word (bounded waits that gave up); 0 when clean.
    int error_status();
    void clear_error();
    size_t cached_bytes() const;

  private:
    SplitOperand *operand(int key, int rows, int K, const MatView &v, int slot);
    void split_into(SplitOperand &op, int rows, int K, const MatView &v);
    void ensure(SplitOperand &op, int rows, int K);
    void free_op(SplitOperand &op);

    int nslices_;
    cudaStream_t st_;
    std::map<int, std::unique_ptr<SplitOperand>> cache_;
    std::map<int, std::unique_ptr<SplitOperand>> dyn_;
    std::map<int, bool> dyn_valid_;
    SplitOperand scratch_[2];
    int *d_err_ = nullptr;
    double *ws_ = nullptr;
    size_t ws_elems_ = 0;
};

// ---- grouped split contractions (batched solve) -------------------------------
// Many systems' operands of one contraction, split into one packed buffer:
// part p's rows occupy rows row0 .. row0 + roundup(rows, 128) of every plane,
// all with the same row pitch kpad (>= every part's K rounded up to 32).
struct PackedSplit {
    void *planes = nullptr;  // __nv_bfloat16*, [nslices][rows][kpad]
    double *scale = nullptr;
    unsigned long long *rmax = nullptr;
    int rows = 0, kpad = 0, nslices = 0;
    size_t bytes = 0;
};
void packed_split_alloc(PackedSplit &op, int rows, int kpad, int nslices);
void packed_split_free(PackedSplit &op);

struct GroupedSplitOperandPart {  // one system's operand view
    MatView v;
    int rows = 0, K = 0, row0 = 0, sys = 0;
};
// Split every active part into `op` (rowmax, then digits); rowc: the views'
// row index is the contiguous one.
void grouped_split_operand_launch(PackedSplit &op, const GroupedSplitOperandPart *d_parts, int nparts,
                                  int max_rows, int max_kpad, bool rowc, const int *active, cudaStream_t st);

struct GroupedSplitPart {  // one system's share of a grouped split contraction
    OutView C;
    const double *scaleA = nullptr, *scaleB = nullptr;  // at the part's first packed row
    double alpha = 0.0, beta = 0.0;
    int M = 0, N = 0, nkb = 0, rowA0 = 0, rowB0 = 0, tiles_m = 0, tiles_n = 0, tile_begin = 0, sys = 0;
};
// Column tile width of grouped launches (64 or 128) for the parts' largest N.
int grouped_split_bn(int max_n);
// C_p = alpha_p A_p B_p^T + beta_p C_p for every active part, one CTA per 128 x bn
// tile (parts[].tile_begin: prefix of tiles_m * tiles_n); no split-K (K < 131072).
void grouped_split_gemm_launch(const PackedSplit &A, const PackedSplit &B, int bn, const GroupedSplitPart *d_parts,
                               int nparts, int total_tiles, const int *active, int *d_err, cudaStream_t st);

// FP64 view -> split operand (S BF16 planes + row scales).
void split_operand_kernel_launch(SplitOperand &op, int rows, int K, const MatView &v, cudaStream_t st);
// C = alpha * A B^T + beta C for split operands with equal kpad and nslices;
// `ws` (ws_elems doubles) holds split-K partial sums; `d_err` the error word.
void split_gemm_launch(const SplitOperand &A, const SplitOperand &B, int M, int N, double alpha, double beta,
                       const OutView &C, double *ws, size_t ws_elems, int *d_err, cudaStream_t st);
// One contraction with temporary split operands and workspace.
void split_gemm_oneshot(int nslices, int M, int N, int K, double alpha, const MatView &A, const MatView &B,
                        double beta, const OutView &C, cudaStream_t st);

}  // namespace ccsd
