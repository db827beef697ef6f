"""GPU tests of the contraction kernels through ccsd_gemm (C ABI) against a
plain PyTorch FP64 reference of the same product.

Tolerances: the FP64 kernel must agree to 1e-13 relative to |A||B|^T; the
split kernel with S BF16 planes represents each operand to 2^-(8S) of its row
maximum and accumulates level 0 exactly, so its error is bounded by
tol_S * (rowmax|A| * rowmax|B| * K) with tol_S = 2^-(8S-3)."""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from ccsd_parallel_gb300 import _abi

pytestmark = pytest.mark.gpu

PREC = {"fp64": 0, "split2": 2, "split3": 3, "split4": 4}


def run_gemm(prec, A, B, Cin=None, alpha=1.0, beta=0.0):
    M, K = A.shape
    N = B.shape[0]
    Cout = torch.zeros(M, N, dtype=torch.float64, device="cuda") if Cin is None else Cin.clone()
    torch.cuda.synchronize()
    rc = _abi.lib().ccsd_gemm(PREC[prec], M, N, K, alpha, C.c_void_p(A.data_ptr()), A.stride(0),
                              C.c_void_p(B.data_ptr()), B.stride(0), beta, C.c_void_p(Cout.data_ptr()),
                              Cout.stride(0), None)
    _abi.check(rc)
    return Cout


def bound(A, B, S):
    ra = A.abs().amax(dim=1, keepdim=True)
    rb = B.abs().amax(dim=1, keepdim=True)
    return (ra @ rb.T) * A.shape[1] * 2.0 ** (-(8 * S - 3))


SHAPES = [(1, 1, 1), (5, 7, 3), (128, 128, 32), (200, 70, 1000), (130, 33, 2500), (300, 300, 5000),
          (1000, 20, 64), (64, 513, 4097), (5000, 1, 300), (1, 700, 9000), (40, 1000, 500)]


# short side <= 16 with a long K: the skinny form (K-split, B staged in shared
# memory), with the short side in M, in N, or a single column
SKINNY = [(2000, 6, 3000), (7, 900, 1200), (240, 1, 100000), (3000, 16, 257), (100, 9, 256), (64, 3, 5000),
          (33, 2, 70000)]


# short side <= 16 with K <= 64 over many rows: the thin form (one thread per row,
# B in shared memory), short side in N or in M
THIN = [(5000, 8, 8), (7, 3000, 64), (300, 16, 1), (100000, 3, 33), (2000, 2, 64)]


@pytest.mark.parametrize("M,N,K", SHAPES + SKINNY + THIN)
def test_fp64_kernel(M, N, K):
    g = torch.Generator(device="cuda").manual_seed(M * 7 + N * 13 + K)
    A = torch.randn(M, K, dtype=torch.float64, device="cuda", generator=g)
    B = torch.randn(N, K, dtype=torch.float64, device="cuda", generator=g)
    C0 = torch.randn(M, N, dtype=torch.float64, device="cuda", generator=g)
    out = run_gemm("fp64", A, B, C0, alpha=0.7, beta=-1.3)
    ref = 0.7 * (A @ B.T) - 1.3 * C0
    scale = 0.7 * (A.abs() @ B.abs().T) + 1.3 * C0.abs()
    assert ((out - ref).abs() <= 1e-13 * scale + 1e-300).all()


@pytest.mark.parametrize("M,N,K", SHAPES)
def test_fp64_dmma_kernel(M, N, K):
    """The tiled FP64 kernel with its inner product on the FP64 tensor pipe
    (mma.sync m8n8k4, ccsd_set_fp64_kernel) holds the same 1e-13 bound."""
    g = torch.Generator(device="cuda").manual_seed(M * 5 + N * 11 + K)
    A = torch.randn(M, K, dtype=torch.float64, device="cuda", generator=g)
    B = torch.randn(N, K, dtype=torch.float64, device="cuda", generator=g)
    C0 = torch.randn(M, N, dtype=torch.float64, device="cuda", generator=g)
    prev = _abi.lib().ccsd_set_fp64_kernel(1)
    try:
        out = run_gemm("fp64", A, B, C0, alpha=0.7, beta=-1.3)
    finally:
        _abi.lib().ccsd_set_fp64_kernel(prev)
    ref = 0.7 * (A @ B.T) - 1.3 * C0
    scale = 0.7 * (A.abs() @ B.abs().T) + 1.3 * C0.abs()
    assert ((out - ref).abs() <= 1e-13 * scale + 1e-300).all()


def test_fp64_kernel_switch_rejects_unknown_kind():
    lib = _abi.lib()
    assert lib.ccsd_set_fp64_kernel(7) == _abi.CCSD_ERR_INVALID_ARG
    prev = lib.ccsd_set_fp64_kernel(1)
    assert lib.ccsd_set_fp64_kernel(prev) == 1


def test_fp64_kernel_beyond_grid_y():
    """N over 65535 column tiles (the CCSDT X3 term's V^3 O columns at nocc=6,
    nvir=40 are 6.1M) runs with the long side in the grid's x dimension."""
    M, N, K = 24, 64 * 65535 + 100, 8
    g = torch.Generator(device="cuda").manual_seed(5)
    A = torch.randn(M, K, dtype=torch.float64, device="cuda", generator=g)
    B = torch.randn(N, K, dtype=torch.float64, device="cuda", generator=g)
    C0 = torch.randn(M, N, dtype=torch.float64, device="cuda", generator=g)
    out = run_gemm("fp64", A, B, C0, alpha=0.7, beta=-1.3)
    ref = 0.7 * (A @ B.T) - 1.3 * C0
    scale = 0.7 * (A.abs() @ B.abs().T) + 1.3 * C0.abs()
    assert ((out - ref).abs() <= 1e-13 * scale + 1e-300).all()


@pytest.mark.parametrize("prec,S", [("split2", 2), ("split3", 3), ("split4", 4)])
@pytest.mark.parametrize("M,N,K", SHAPES)
def test_split_kernel(prec, S, M, N, K):
    g = torch.Generator(device="cuda").manual_seed(M * 5 + N * 3 + K + S)
    A = torch.randn(M, K, dtype=torch.float64, device="cuda", generator=g)
    B = torch.randn(N, K, dtype=torch.float64, device="cuda", generator=g)
    out = run_gemm(prec, A, B)
    ref = A @ B.T
    err = (out - ref).abs()
    assert (err <= bound(A, B, S)).all(), float((err / bound(A, B, S)).max())


def test_split_alpha_beta_and_wide_dynamic_range():
    g = torch.Generator(device="cuda").manual_seed(3)
    M, N, K = 256, 96, 3000
    A = torch.randn(M, K, dtype=torch.float64, device="cuda", generator=g)
    A *= torch.logspace(-6, 3, M, device="cuda", dtype=torch.float64)[:, None]
    B = torch.randn(N, K, dtype=torch.float64, device="cuda", generator=g)
    A[7] = 0.0
    C0 = torch.randn(M, N, dtype=torch.float64, device="cuda", generator=g)
    out = run_gemm("split4", A, B, C0, alpha=-2.0, beta=0.5)
    ref = -2.0 * (A @ B.T) + 0.5 * C0
    assert ((out - ref).abs() <= 2.0 * bound(A, B, 4) + 1e-15 * C0.abs()).all()
    assert torch.equal(out[7], 0.5 * C0[7])


def test_split_level0_is_exact_for_integer_operands():
    """Integer operands with a row maximum of 127 get the row scale 2^7 and sit
    entirely in plane 0, so the result is the exact integer product (no FP32
    rounding over long K).  (A row maximum of exactly 128 would get the scale
    2^8 and spill the odd integers into plane 1.)"""
    g = torch.Generator(device="cuda").manual_seed(11)
    M, N, K = 160, 48, 20000
    A = torch.randint(-127, 128, (M, K), generator=g, device="cuda").to(torch.float64)
    A[:, 0] = 127.0
    B = torch.randint(-127, 128, (N, K), generator=g, device="cuda").to(torch.float64)
    B[:, 0] = -127.0
    out = run_gemm("split2", A, B)
    ref = A @ B.T
    assert torch.equal(out, ref)


def test_fp64_solve_with_dmma_matches_dfma():
    """A whole FP64 CCSD solve (every view orientation of the tiled kernel) with
    the DMMA inner product: same iteration count and E_corr within 1e-12 of the
    DFMA solve, T2 within 1e-11."""
    import ccsd_parallel_gb300 as cg
    o, v, q = 6, 40, 120
    fock, b = cg.make_synthetic(o, v, q, 11)
    out = []
    lib = _abi.lib()
    for kind in (0, 1):
        prev = lib.ccsd_set_fp64_kernel(kind)
        try:
            with cg.Solver(fock, o, df=b, precision="fp64", energy_tol=1e-12) as s:
                out.append(s.solve())
        finally:
            lib.ccsd_set_fp64_kernel(prev)
    a, d = out
    assert a["converged"] and d["converged"]
    assert a["iterations"] == d["iterations"]
    assert abs(a["e_corr"] - d["e_corr"]) < 1e-12
    assert np.abs(a["t2"] - d["t2"]).max() < 1e-11
