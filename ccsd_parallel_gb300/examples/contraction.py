"""Time one contraction of the engine through the C ABI (ccsd_gemm).

    python -m ccsd_parallel_gb300.examples.contraction --M 7200 --N 7200 --K 7200 --precision 3 --repeat 3

C[M][N] = A[M][K] B[N][K]^T + C with row-major FP64 device operands (seeded
normal entries), the shape of the o v x o v x o v ring contractions of a CCSD
update at o v = 7200.  Each call splits both operands and runs the
contraction; the CUDA-event time of each call and its algorithmic rate
(2 M N K flop) are printed, one line per call.
"""
from __future__ import annotations

import argparse
import ctypes as C

import torch

from ccsd_parallel_gb300 import _abi


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--M", type=int, default=7200)
    ap.add_argument("--N", type=int, default=7200)
    ap.add_argument("--K", type=int, default=7200)
    ap.add_argument("--precision", type=int, default=3, help="0 = FP64, 2/3/4 = split BF16 planes")
    ap.add_argument("--repeat", type=int, default=3)
    ap.add_argument("--fp64-kernel", choices=("dfma", "dmma"), default="dfma",
                    help="inner product of the FP64 tiled kernel (precision 0)")
    a = ap.parse_args()
    g = torch.Generator(device="cuda").manual_seed(0)
    A = torch.randn(a.M, a.K, dtype=torch.float64, device="cuda", generator=g)
    B = torch.randn(a.N, a.K, dtype=torch.float64, device="cuda", generator=g)
    Cm = torch.zeros(a.M, a.N, dtype=torch.float64, device="cuda")
    lib = _abi.lib()
    lib.ccsd_set_fp64_kernel(1 if a.fp64_kernel == "dmma" else 0)
    for r in range(a.repeat):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        rc = lib.ccsd_gemm(a.precision, a.M, a.N, a.K, 1.0, C.c_void_p(A.data_ptr()), a.K, C.c_void_p(B.data_ptr()),
                           a.K, 1.0, C.c_void_p(Cm.data_ptr()), a.N, None)
        e1.record()
        torch.cuda.synchronize()
        _abi.check(rc)
        ms = e0.elapsed_time(e1)
        print(f"call {r}: {ms:.3f} ms (split + contraction), {2.0 * a.M * a.N * a.K / ms / 1e9:.1f} TFLOP/s")


if __name__ == "__main__":
    main()
