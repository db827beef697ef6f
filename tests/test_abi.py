"""CPU tests of the C ABI: the library loads without a GPU, exports every
function include/ccsd_gb300.h declares, and its host-only helpers agree with
the oracle.  No compute call runs here."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from ccsd_parallel_gb300 import _abi
from oracle import synthetic as syn

ROOT = Path(__file__).resolve().parent.parent


def _declared():
    names = []
    for h in sorted((ROOT / "include").glob("*.h")):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names += re.findall(r"^\s*(?:int|double|void)\s*\*?\s*(ccsd_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol():
    lib = _abi.lib()
    names = _declared()
    assert "ccsd_create" in names and "ccsd_solve" in names
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # the ctypes table covers the same set
    assert set(names) <= set(_abi.SIGNATURES)


def test_struct_layouts_match_header_sizes():
    assert C.sizeof(_abi.Problem) == 6 * 4 + 4 * 8 + 8  # nfrozen (int32) padded to 8
    assert C.sizeof(_abi.Options) == 2 * 8 + 8 * 4 + 8 + 2 * 8 + 8  # + t1_start, t2_start, variant (padded)
    assert C.sizeof(_abi.Result) == 2 * 8 + 2 * 4 + 4 * 8 + 2 * 4 + 8


def test_struct_layouts_match_compiled_header(tmp_path):
    """Size and every field offset of the ctypes mirrors equal what a C
    compiler makes of include/ccsd_gb300.h."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    structs = {"ccsd_problem": _abi.Problem, "ccsd_options": _abi.Options, "ccsd_result": _abi.Result,
               "ccsd_grad": _abi.Grad}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "ccsd_gb300.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for f, _ in py._fields_:
            lines.append(f'  printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c11", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    got = {}
    for line in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines():
        s, f, val = line.split()
        got[(s, f)] = int(val)
    for cname, py in structs.items():
        assert got[(cname, "size")] == C.sizeof(py), cname
        for f, _ in py._fields_:
            assert got[(cname, f)] == getattr(py, f).offset, (cname, f)


def test_default_options_follow_reference_rules():
    o = _abi.Options()
    assert _abi.lib().ccsd_default_options(C.byref(o)) == 0
    assert o.energy_tol == 1e-10 and o.max_iter == 999 and o.diis_size == 0
    assert o.precision == _abi.CCSD_PREC_FP64


def test_flop_count_formula():
    f = _abi.lib().ccsd_flops_per_update(24, 300)
    o, v = 24.0, 300.0
    assert f == pytest.approx(2 * o**2 * v**4 + 4 * o**4 * v**2 + 8 * o**3 * v**3)
    assert f == pytest.approx(1.24e13, rel=0.02)


def test_frozen_core_count_follows_reference_rule():
    """One frozen spatial orbital per atom with 2 < Z < 11, none for H, He or
    beyond Ne (Freeze_How_Meny_Orbitals, ccsd_memory_optimized.cpp:5203-5231),
    counted per atom."""
    import ccsd_parallel_gb300 as cg
    assert cg.frozen_core_count([8.0, 1.0, 1.0]) == 1
    assert cg.frozen_core_count([6.0, 8.0, 8.0]) == 3
    assert cg.frozen_core_count([1.0, 2.0, 11.0, 17.0]) == 0
    assert cg.frozen_core_count([3.0, 10.0]) == 2
    assert cg.frozen_core_count([]) == 0
    assert _abi.lib().ccsd_frozen_core_count(None, -1) == _abi.CCSD_ERR_INVALID_ARG
    assert _abi.lib().ccsd_frozen_core_count(None, 2) == _abi.CCSD_ERR_INVALID_ARG


def test_library_generator_matches_oracle_generator():
    o, v, q, seed = 3, 9, 7, 99
    n = o + v
    fock = np.zeros((n, n))
    b = np.zeros((q, n, n))
    rc = _abi.lib().ccsd_make_synthetic(o, v, q, seed, fock.ctypes.data_as(C.POINTER(C.c_double)),
                                        b.ctypes.data_as(C.POINTER(C.c_double)))
    assert rc == 0
    f_ref, b_ref = syn.make_system(o, v, q, seed)
    np.testing.assert_allclose(fock, f_ref, rtol=0, atol=1e-15)
    np.testing.assert_allclose(b, b_ref, rtol=1e-14, atol=1e-17)
    assert np.array_equal(b, b.transpose(0, 2, 1))


def test_invalid_arguments_fail_without_compute():
    lib = _abi.lib()
    h = C.c_void_p()
    assert lib.ccsd_create(None, None, C.byref(h)) == _abi.CCSD_ERR_INVALID_ARG
    assert "NULL" in _abi.last_error()
    assert lib.ccsd_solve(None, None) == _abi.CCSD_ERR_INVALID_ARG
    assert lib.ccsd_make_synthetic(0, 5, 3, 1, None, None) == _abi.CCSD_ERR_INVALID_ARG
    assert lib.ccsd_destroy(None) == 0


def test_no_cpu_path_when_no_device():
    """With no GPU visible, ccsd_create refuses (no silent CPU fallback)."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    fock, b = syn.make_system(2, 4, 5, 1)
    p = _abi.Problem()
    p.nocc, p.nvir, p.integral_kind, p.naux = 2, 4, _abi.CCSD_INTS_DF, 5
    fock = np.ascontiguousarray(fock)
    b = np.ascontiguousarray(b)
    p.fock = fock.ctypes.data_as(C.POINTER(C.c_double))
    p.df = b.ctypes.data_as(C.POINTER(C.c_double))
    h = C.c_void_p()
    rc = _abi.lib().ccsd_create(C.byref(p), None, C.byref(h))
    assert rc == _abi.CCSD_ERR_NO_DEVICE
    assert "no CPU path" in _abi.last_error()


def test_integrals_have_no_cpu_path():
    """ccsd_ao_integrals refuses without a GPU as well."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    import ccsd_parallel_gb300 as cg
    d = np.load(ROOT / "tests" / "golden" / "ints_h2o_sto3g.npz")
    with pytest.raises(cg.CCSDError) as ei:
        cg.ao_integrals(d)
    assert ei.value.code == _abi.CCSD_ERR_NO_DEVICE


def test_batched_solve_refuses_restart_amplitudes():
    """t1_start / t2_start belong to single solves; the batched entry refuses them
    before touching a device."""
    p = _abi.Problem()
    p.nocc, p.nvir, p.integral_kind, p.naux = 2, 4, _abi.CCSD_INTS_DF, 5
    fock, b = syn.make_system(2, 4, 5, 1)
    fock, b = np.ascontiguousarray(fock), np.ascontiguousarray(b)
    p.fock = fock.ctypes.data_as(C.POINTER(C.c_double))
    p.df = b.ctypes.data_as(C.POINTER(C.c_double))
    o = _abi.Options()
    _abi.lib().ccsd_default_options(C.byref(o))
    t2 = np.zeros(2 * 2 * 4 * 4)
    o.t2_start = t2.ctypes.data_as(C.POINTER(C.c_double))
    probs = (C.POINTER(_abi.Problem) * 1)(C.pointer(p))
    res = (_abi.Result * 1)()
    rc = _abi.lib().ccsd_solve_batched(probs, 1, C.byref(o), res)
    assert rc == _abi.CCSD_ERR_INVALID_ARG
    assert "single solves" in _abi.last_error()
