// Element-wise FP64 helpers that spend as few FP64-pipe instructions as the
// operands allow.  On this part the FP64 pipe runs at 1/64 of the FP32 rate,
// about 0.6e12 instructions/s against 0.85e12 doubles/s of HBM bandwidth, so an
// element-wise pass that does more than about one FP64 add, multiply or FMA per
// double it moves is bound by that pipe, not by memory.
#pragma once

#include <cuda_runtime.h>

namespace ccsd {

// alpha x + beta y, rounded as fma(beta, y, alpha x); alpha = 1 or beta = 0 or 1
// skip the operations they make trivial (the results are identical).  The case is
// classified once per thread (axpby_mode: the comparisons are FP64 instructions too)
// and applied per element (axpby_apply).
enum AxpbyMode { kAxX, kAxAX, kAxXpY, kAxXpBY, kAxGen, kAxY, kAxBY, kAxZero };
__host__ __device__ __forceinline__ int axpby_mode(double alpha, double beta) {
    if (beta == 0.0) return alpha == 1.0 ? kAxX : (alpha == 0.0 ? kAxZero : kAxAX);
    if (alpha == 0.0) return beta == 1.0 ? kAxY : kAxBY;
    if (alpha == 1.0) return beta == 1.0 ? kAxXpY : kAxXpBY;
    return kAxGen;
}
__device__ __forceinline__ double axpby_apply(int mode, double alpha, double x, double beta, double y) {
    switch (mode) {
        case kAxX: return x;
        case kAxAX: return alpha * x;
        case kAxXpY: return x + y;
        case kAxXpBY: return fma(beta, y, x);
        case kAxY: return y;
        case kAxBY: return beta * y;
        case kAxZero: return 0.0;
        default: return fma(beta, y, alpha * x);
    }
}
__device__ __forceinline__ bool axpby_reads_x(int mode) { return mode != kAxY && mode != kAxBY && mode != kAxZero; }
__device__ __forceinline__ bool axpby_reads_y(int mode) { return mode >= kAxXpY && mode <= kAxBY; }

// x 2^k (|k| small) by 32-bit integer arithmetic on the exponent field of the high
// word when x and the result are normal numbers; the FP64 product otherwise (zero,
// subnormal, inf, NaN).  (64-bit integer arithmetic is avoided in these helpers: ncu
// counts it on the FP64 pipe here.)
__device__ __forceinline__ double mul_pow2(double x, int k) {
    const int hi = __double2hiint(x);
    const int e = (hi >> 20) & 0x7FF;
    if (e > 0 && e < 0x7FF && e + k > 0 && e + k < 0x7FF) return __hiloint2double(hi + (k << 20), __double2loint(x));
    return x * __hiloint2double((1023 + k) << 20, 0);
}

}  // namespace ccsd
