// Element-wise FP64 helpers that spend as few FP64-pipe instructions as the
// operands allow.  On this part the FP64 pipe runs at 1/64 of the FP32 rate,
// about 0.6e12 instructions/s against 0.85e12 doubles/s of HBM bandwidth, so an
// element-wise pass that does more than about one FP64 add, multiply or FMA per
// double it moves is bound by that pipe, not by memory.
#pragma once

#include <cuda_runtime.h>

namespace ccsd {

// alpha x + beta y, rounded as fma(beta, y, alpha x); alpha = 1 or beta = 0 or 1
// skip the operations they make trivial (the results are identical)
__device__ __forceinline__ double axpby_el(double alpha, double x, double beta, double y) {
    if (beta == 0.0) return alpha == 1.0 ? x : (alpha == 0.0 ? 0.0 : alpha * x);
    if (alpha == 0.0) return beta == 1.0 ? y : beta * y;
    if (alpha == 1.0) return beta == 1.0 ? x + y : fma(beta, y, x);
    return fma(beta, y, alpha * x);
}

// x 2^k (|k| small) by integer arithmetic on the exponent field when x and the
// result are normal numbers; the FP64 product otherwise (zero, subnormal, inf, NaN)
__device__ __forceinline__ double mul_pow2(double x, int k) {
    const long long b = __double_as_longlong(x);
    const int e = (int)((b >> 52) & 0x7FF);
    if (e > 0 && e < 0x7FF && e + k > 0 && e + k < 0x7FF) return __longlong_as_double(b + ((long long)k << 52));
    return x * __longlong_as_double((long long)(1023 + k) << 52);
}

}  // namespace ccsd
