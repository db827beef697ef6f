// Split-precision contraction engine on the sm_103a tensor cores.
//
// An FP64 operand x (one row of A or B) is written as
//     x = s * 2^-7 * (P0 + P1 + ... + P_{S-1}),  s = 2^ceil(log2 max|row|),
// where P0 = rint(x/s * 2^7) is an integer in [-128, 128] and every further
// plane carries the next 8 bits of the remainder, pre-scaled by 2^-8 per
// plane.  All planes are exact in BF16.  tcgen05.mma (kind::f16, BF16 in,
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
#include <vector>

#include "common.h"

namespace ccsd {

// Split form of an M x K operand: S planes of [rows_pad][kpad] BF16 (K-major)
// plus one FP64 scale per row.
struct SplitOperand {
    void *planes = nullptr;  // __nv_bfloat16*
    double *scale = nullptr;
    int rows = 0, rows_pad = 0, K = 0, kpad = 0, nslices = 0;
    size_t bytes = 0;
    alignas(64) unsigned char tmap[128];  // CUtensorMap (2-D, over all planes)
};

class SplitEngine {
  public:
    SplitEngine(int nslices, cudaStream_t st);
    ~SplitEngine();
    void set_stream(cudaStream_t st) { st_ = st; }
    int nslices() const { return nslices_; }
    // C(m,n) = alpha * sum_k A(m,k) B(n,k) + beta C(m,n) on the tensor cores.
    void gemm(int M, int N, int K, double alpha, const MatView &A, const MatView &B, double beta,
              const OutView &C, int cache_a, int cache_b);
    // Device error word (bounded waits that gave up); 0 when clean.
    int error_status();
    size_t cached_bytes() const;

  private:
    SplitOperand *operand(int key, int rows, int K, const MatView &v, int slot);
    void split_into(SplitOperand &op, int rows, int K, const MatView &v);
    void ensure(SplitOperand &op, int rows, int K);
    void free_op(SplitOperand &op);

    int nslices_;
    cudaStream_t st_;
    std::map<int, std::unique_ptr<SplitOperand>> cache_;
    SplitOperand scratch_[2];
    int *d_err_ = nullptr;
};

// Raw launch used by the engine and by the C-ABI test entry points.
// A and B are split operands with the same kpad and nslices.
void split_gemm_launch(const SplitOperand &A, const SplitOperand &B, int M, int N, double alpha,
                       double beta, const OutView &C, int *d_err, cudaStream_t st);
void split_operand_kernel_launch(SplitOperand &op, int rows, int K, const MatView &v,
                                 cudaStream_t st);
bool encode_tmap(SplitOperand &op, int box_rows);

}  // namespace ccsd
