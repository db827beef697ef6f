"""GPU test of ccsd_gemm_noalloc, the contraction entry point that allocates
no device memory (for callers whose device memory is owned by another
allocator, or who cannot take cudaFree's device-wide synchronisation).

It runs through the C ABI and is checked against the allocating entry point
ccsd_gemm on the same inputs, within the split kernel's error bound used by
the other kernel tests, on two calls in a row (the second call reuses the
static scratch array the first call left behind).  This file is collected
last so a failure here cannot hide the result of any other test."""
import ctypes as C

import pytest

torch = pytest.importorskip("torch")

from ccsd_parallel_gb300 import _abi

pytestmark = pytest.mark.gpu


def _call(name, prec, A, B, Cout, alpha=1.0, beta=0.0):
    M, K = A.shape
    N = B.shape[0]
    torch.cuda.synchronize()
    rc = getattr(_abi.lib(), name)(prec, M, N, K, alpha, C.c_void_p(A.data_ptr()), A.stride(0),
                                   C.c_void_p(B.data_ptr()), B.stride(0), beta,
                                   C.c_void_p(Cout.data_ptr()), Cout.stride(0), None)
    return rc


def _bound(A, B, S):
    ra = A.abs().amax(dim=1, keepdim=True)
    rb = B.abs().amax(dim=1, keepdim=True)
    return (ra @ rb.T) * A.shape[1] * 2.0 ** (-(8 * S - 3))


@pytest.mark.parametrize("S", [2, 3, 4])
def test_noalloc_matches_allocating_entry_point_twice(S):
    g = torch.Generator(device="cuda").manual_seed(100 + S)
    shapes = [(300, 200, 3000), (70, 500, 1500)]  # the second exercises the transposed roles
    for (M, N, K) in shapes:
        for call in range(2):
            A = torch.randn(M, K, dtype=torch.float64, device="cuda", generator=g)
            B = torch.randn(N, K, dtype=torch.float64, device="cuda", generator=g)
            C0 = torch.randn(M, N, dtype=torch.float64, device="cuda", generator=g)
            ref = C0.clone()
            out = C0.clone()
            assert _call("ccsd_gemm", S, A, B, ref, alpha=0.5, beta=-1.0) == 0, _abi.last_error()
            assert _call("ccsd_gemm_noalloc", S, A, B, out, alpha=0.5, beta=-1.0) == 0, _abi.last_error()
            tol = 0.5 * _bound(A, B, S)
            assert ((out - ref).abs() <= tol).all(), (M, N, K, call, float(((out - ref).abs() / tol).max()))
            exact = 0.5 * (A @ B.T) - C0
            assert ((out - exact).abs() <= tol).all()


def test_noalloc_rejects_oversized_operands():
    A = torch.zeros(4096, 4096, dtype=torch.float64, device="cuda")
    B = torch.zeros(4096, 4096, dtype=torch.float64, device="cuda")
    out = torch.zeros(4096, 4096, dtype=torch.float64, device="cuda")
    rc = _call("ccsd_gemm_noalloc", 3, A, B, out)
    assert rc == _abi.CCSD_ERR_INVALID_ARG
    assert "64 MiB" in _abi.last_error()
    rc = _call("ccsd_gemm_noalloc", 0, A[:8, :8], B[:8, :8], out[:8, :8])
    assert rc == _abi.CCSD_ERR_INVALID_ARG


@pytest.mark.parametrize("name,prec", [("ccsd_gemm", 0), ("ccsd_gemm", 3), ("ccsd_gemm_noalloc", 3)])
def test_empty_contraction_scales_c(name, prec):
    """K = 0: nothing is contracted and C becomes beta * C (beta = 0 clears C,
    NaN included; beta = 1 leaves it untouched)."""
    dummy = torch.zeros(1, dtype=torch.float64, device="cuda")  # A and B are never read
    for beta in (0.0, 1.0, -2.5):
        C0 = torch.randn(40, 30, dtype=torch.float64, device="cuda")
        C0[0, 0] = float("nan") if beta == 0.0 else C0[0, 0]
        out = C0.clone()
        M, N = 40, 30
        torch.cuda.synchronize()
        rc = getattr(_abi.lib(), name)(prec, M, N, 0, 0.7, C.c_void_p(dummy.data_ptr()), 0,
                                       C.c_void_p(dummy.data_ptr()), 0, beta, C.c_void_p(out.data_ptr()), N, None)
        assert rc == 0, _abi.last_error()
        expect = torch.zeros_like(C0) if beta == 0.0 else beta * C0
        assert torch.equal(out, expect)
