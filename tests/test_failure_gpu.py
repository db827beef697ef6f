"""The device-side failure path, exercised without a GPU fault.

Every mbarrier wait of the split-precision kernel is bounded; one that gives
up sets the error word, stops the kernel's other roles, lets in-flight TMA
loads land and frees TMEM, and the host reports CCSD_ERR_TIMEOUT.  The test
makes one wait run out on purpose (ccsd_debug_stall_split_mma: the MMA thread
waits on an mbarrier that nothing arrives at, bounded by 2 ms), checks the
status through ccsd_gemm and ccsd_solve, and then checks that the same
context, and the same solver handle, compute correctly again."""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import ccsd_parallel_gb300 as cg
from ccsd_parallel_gb300 import _abi

pytestmark = pytest.mark.gpu

STALL_NS = 2_000_000


def _gemm(prec, A, B, out):
    M, K = A.shape
    N = B.shape[0]
    torch.cuda.synchronize()
    return _abi.lib().ccsd_gemm(prec, M, N, K, 1.0, C.c_void_p(A.data_ptr()), K, C.c_void_p(B.data_ptr()), K,
                                0.0, C.c_void_p(out.data_ptr()), N, None)


def test_stalled_wait_reports_timeout_and_the_context_recovers():
    lib = _abi.lib()
    g = torch.Generator(device="cuda").manual_seed(3)
    A = torch.randn(256, 512, dtype=torch.float64, device="cuda", generator=g)
    B = torch.randn(192, 512, dtype=torch.float64, device="cuda", generator=g)
    out = torch.zeros(256, 192, dtype=torch.float64, device="cuda")
    fock, b = cg.make_synthetic(8, 60, 120, 11)
    s = cg.Solver(fock, 8, df=b, precision="split3", fixed_iterations=3)
    assert lib.ccsd_debug_stall_split_mma(STALL_NS) == 0
    try:
        assert _gemm(3, A, B, out) == _abi.CCSD_ERR_TIMEOUT
        assert "bounded device wait" in _abi.last_error()
        with pytest.raises(cg.CCSDError) as ei:
            s.solve()
        assert ei.value.code == _abi.CCSD_ERR_TIMEOUT
    finally:
        assert lib.ccsd_debug_stall_split_mma(0) == 0
    # the context is intact: the same contraction and the same handle now succeed
    assert _gemm(3, A, B, out) == 0, _abi.last_error()
    bound = (A.abs().amax(1, keepdim=True) @ B.abs().amax(1, keepdim=True).T) * 512 * 2.0 ** -21
    assert ((out - A @ B.T).abs() <= bound).all()
    r = s.solve()
    s.close()
    r64 = cg.solve(fock, 8, df=b, fixed_iterations=3)
    np.testing.assert_allclose(r["energies"], r64["energies"], rtol=0, atol=1e-9)
