"""ctypes binding of ``include/ccsd_gb300.h`` (the C ABI of the CUDA library).

The library is the in-tree ``_lib/libccsd_gb300.so``.  Loading it needs no GPU;
every compute entry point fails with ``CCSD_ERR_NO_DEVICE`` when no device is
present (there is no CPU path).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libccsd_gb300.so"

CCSD_OK = 0
CCSD_ERR_INVALID_ARG = -1
CCSD_ERR_CUDA = -2
CCSD_ERR_OUT_OF_MEMORY = -3
CCSD_ERR_DIVERGED = -4
CCSD_ERR_NO_DEVICE = -5
CCSD_BASIS_ACCURATE_BOYS = 1
CCSD_ERR_TIMEOUT = -6
CCSD_ERR_UNSUPPORTED = -7
CCSD_ERR_NOT_CONVERGED = -8

CCSD_INTS_MO_DENSE = 0
CCSD_INTS_DF = 1
CCSD_INTS_AO_DENSE = 2
CCSD_INTS_SO_ANTISYM = 3

CCSD_METHOD_CCSD = 0
CCSD_METHOD_CCSDT1A = 1
CCSD_METHOD_CCSDT1B = 2
CCSD_METHOD_CCSDT2 = 3
CCSD_METHOD_CCSDT3 = 4
CCSD_METHOD_CCSDT4 = 5
CCSD_METHOD_CCSDT = 6
CCSD_VARIANT_CCSD = 0
CCSD_VARIANT_MEMORY_OPTIMIZED = 1

CCSD_PREC_FP64 = 0
CCSD_PREC_SPLIT2 = 2
CCSD_PREC_SPLIT3 = 3
CCSD_PREC_SPLIT4 = 4

_dp = C.POINTER(C.c_double)


class Problem(C.Structure):
    _fields_ = [
        ("nocc", C.c_int32), ("nvir", C.c_int32), ("integral_kind", C.c_int32),
        ("naux", C.c_int32), ("nao", C.c_int32), ("device_inputs", C.c_int32),
        ("fock", _dp), ("eri", _dp), ("df", _dp), ("mo_coeff", _dp), ("nfrozen", C.c_int32),
    ]


class Basis(C.Structure):
    _fields_ = [
        ("natoms", C.c_int32), ("nbf", C.c_int32), ("maxprim", C.c_int32), ("flags", C.c_int32),
        ("Z", _dp), ("R", _dp), ("atom", C.POINTER(C.c_int32)), ("powers", C.POINTER(C.c_int32)),
        ("nprim", C.POINTER(C.c_int32)), ("alpha", _dp), ("coef", _dp),
    ]


class ScfResult(C.Structure):
    _fields_ = [
        ("e_hf", C.c_double), ("e_nuc", C.c_double), ("iterations", C.c_int32), ("converged", C.c_int32),
        ("eps", _dp), ("C", _dp), ("eri", _dp), ("stream", C.c_void_p),
    ]


class UhfResult(C.Structure):
    _fields_ = [
        ("e_uhf", C.c_double), ("e_nuc", C.c_double), ("iterations", C.c_int32), ("converged", C.c_int32),
        ("eps_up", _dp), ("eps_down", _dp), ("C_up", _dp), ("C_down", _dp), ("seed", C.c_uint64),
        ("stream", C.c_void_p),
    ]


class Incar(C.Structure):
    _fields_ = [
        ("basis_set", C.c_char * 64), ("method", C.c_char * 32), ("convergance_criteria", C.c_double),
        ("freeze_core", C.c_int32), ("relax_pos", C.c_int32), ("use_angstrom", C.c_int32),
        ("print_stuffies", C.c_int32), ("natoms", C.c_int32), ("nbf", C.c_int32), ("maxprim", C.c_int32),
        ("n_electrons", C.c_int32), ("nfrozen", C.c_int32), ("capacity_atoms", C.c_int32),
        ("capacity_bf", C.c_int32), ("capacity_prim", C.c_int32), ("Z", _dp), ("R", _dp),
        ("atom", C.POINTER(C.c_int32)), ("powers", C.POINTER(C.c_int32)), ("nprim", C.POINTER(C.c_int32)),
        ("alpha", _dp), ("coef", _dp),
    ]


class IncarResult(C.Structure):
    _fields_ = [
        ("energy", C.c_double), ("e_hf", C.c_double), ("e_corr", C.c_double), ("scf_iterations", C.c_int32),
        ("cc_iter", C.c_int32), ("method", C.c_int32), ("nbf", C.c_int32),
    ]


class Options(C.Structure):
    _fields_ = [
        ("energy_tol", C.c_double), ("residual_tol", C.c_double), ("max_iter", C.c_int32),
        ("fixed_iterations", C.c_int32), ("diis_size", C.c_int32), ("diis_start", C.c_int32),
        ("precision", C.c_int32), ("verbose", C.c_int32), ("profile", C.c_int32),
        ("method", C.c_int32), ("stream", C.c_void_p), ("t1_start", _dp), ("t2_start", _dp),
        ("variant", C.c_int32),
    ]


class Result(C.Structure):
    _fields_ = [
        ("e_corr", C.c_double), ("residual_norm", C.c_double), ("iterations", C.c_int32),
        ("converged", C.c_int32), ("t1", _dp), ("t2", _dp), ("energy_history", _dp),
        ("update_ms", _dp), ("history_capacity", C.c_int32), ("history_len", C.c_int32),
        ("flops_per_update", C.c_double),
    ]


class Grad(C.Structure):
    _fields_ = [
        ("d_fock", _dp), ("d_eri", _dp), ("d_df", _dp), ("d_mo_coeff", _dp), ("lambda1", _dp),
        ("lambda2", _dp), ("tol", C.c_double), ("max_iter", C.c_int32), ("iterations", C.c_int32),
        ("residual_norm", C.c_double), ("e_corr", C.c_double),
    ]


# Every function the header declares, with its ctypes signature.
SIGNATURES = {
    "ccsd_default_options": (C.c_int, [C.POINTER(Options)]),
    "ccsd_create": (C.c_int, [C.POINTER(Problem), C.POINTER(Options), C.POINTER(C.c_void_p)]),
    "ccsd_solve": (C.c_int, [C.c_void_p, C.POINTER(Result)]),
    "ccsd_lambda_grad": (C.c_int, [C.c_void_p, C.POINTER(Problem), C.POINTER(Grad)]),
    "ccsd_set_options": (C.c_int, [C.c_void_p, C.POINTER(Options)]),
    "ccsd_destroy": (C.c_int, [C.c_void_p]),
    "ccsd_last_error": (C.c_int, [C.c_char_p, C.c_size_t]),
    "ccsd_profile_report": (C.c_int, [C.c_void_p, C.c_char_p, C.c_size_t]),
    "ccsd_flops_per_update": (C.c_double, [C.c_int32, C.c_int32]),
    "ccsd_frozen_core_count": (C.c_int, [_dp, C.c_int32]),
    "ccsd_incar_parse": (C.c_int, [C.c_char_p, C.c_char_p, C.POINTER(Incar)]),
    "ccsd_incar_run": (C.c_int, [C.c_char_p, C.c_char_p, C.c_int32, C.POINTER(IncarResult)]),
    "ccsd_uhf": (C.c_int, [C.POINTER(Basis), C.c_int32, C.c_int32, C.c_double, C.c_int32, C.POINTER(UhfResult)]),
    "ccsd_rhf": (C.c_int, [C.POINTER(Basis), C.c_int32, C.c_double, C.c_int32, C.POINTER(ScfResult)]),
    "ccsd_ao_integrals": (C.c_int, [C.POINTER(Basis), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                    C.POINTER(C.c_double), C.c_int32, C.c_void_p]),
    "ccsd_make_synthetic": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.c_uint64, _dp, _dp]),
    "ccsd_gemm": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_double, C.c_void_p,
                            C.c_int64, C.c_void_p, C.c_int64, C.c_double, C.c_void_p, C.c_int64,
                            C.c_void_p]),
    "ccsd_batch_create": (C.c_int, [C.POINTER(C.POINTER(Problem)), C.c_int32, C.POINTER(Options),
                                    C.POINTER(C.c_void_p)]),
    "ccsd_batch_solve": (C.c_int, [C.c_void_p, C.POINTER(Result)]),
    "ccsd_batch_report": (C.c_int, [C.c_void_p, C.c_char_p, C.c_size_t]),
    "ccsd_batch_destroy": (C.c_int, [C.c_void_p]),
    "ccsd_solve_batched": (C.c_int, [C.POINTER(C.POINTER(Problem)), C.c_int32, C.POINTER(Options),
                                     C.POINTER(Result)]),
    "ccsd_gemm_noalloc": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_double, C.c_void_p,
                                    C.c_int64, C.c_void_p, C.c_int64, C.c_double, C.c_void_p, C.c_int64,
                                    C.c_void_p]),
    "ccsd_debug_stall_split_mma": (C.c_int, [C.c_uint64]),
    "ccsd_set_fp64_kernel": (C.c_int, [C.c_int32]),
}

_lib = None


def lib():
    """Load the library once; raise loudly when it is missing (no fallback)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(
                f"CUDA library {LIB_PATH} is missing: run __graft_entry__.build() "
                "(this package has no CPU fallback)")
        h = C.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            f = getattr(h, name)
            f.restype = res
            f.argtypes = args
        _lib = h
    return _lib


def last_error() -> str:
    buf = C.create_string_buffer(4096)
    lib().ccsd_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


class CCSDError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"ccsd error {code}: {msg}")
        self.code = code


def check(rc: int):
    if rc != CCSD_OK:
        raise CCSDError(rc, last_error())
    return rc
