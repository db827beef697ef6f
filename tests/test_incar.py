"""The INCAR front end's parsing (ccsd_incar_parse, host only): the reference's
INCAR keywords and atom lines (main.cpp:83-298) and a Gaussian94 basis expanded
to the arrays the reference's integral engine receives (Cartesian order and
primitive normalisation of Normalize_small_c), checked against the reference's
own arrays in tests/golden/ints_*.npz; the reader's hazards fixed."""
from pathlib import Path

import numpy as np
import pytest

import ccsd_parallel_gb300 as cg
from ccsd_parallel_gb300 import _abi
from incar_util import g94_from_fixture, incar_text

GOLD = Path(__file__).parent / "golden"
CASES = ["h2o_sto3g", "nh3_sto3g", "h2o_631g", "h2o_ccpvdz", "o_ccpvtz"]


@pytest.mark.parametrize("name", CASES)
def test_basis_expansion_matches_reference(name):
    d = np.load(GOLD / f"ints_{name}.npz")
    p = cg.parse_incar(incar_text(d, "CCSD", -10), g94_from_fixture(d))
    np.testing.assert_array_equal(p["atom"], d["atom"])
    np.testing.assert_array_equal(p["powers"], d["powers"])
    np.testing.assert_array_equal(p["nprim"], d["nprim"])
    mp = p["alpha"].shape[1]
    np.testing.assert_array_equal(p["alpha"], d["alpha"][:, :mp])
    np.testing.assert_allclose(p["coef"], d["coef"][:, :mp], rtol=1e-14, atol=0)
    np.testing.assert_array_equal(p["Z"], d["Z"])
    np.testing.assert_array_equal(p["R"], d["R"])
    assert p["n_electrons"] == int(np.sum(d["Z"]))
    assert p["method"] == "CCSD" and p["tol"] == pytest.approx(1e-10, rel=1e-15)


def test_incar_reader_hazards():
    d = np.load(GOLD / "ints_h2o_sto3g.npz")
    basis = g94_from_fixture(d)
    # a keyword inside a comment or another value does not count; blanks of any length
    text = ("# Method HF would be taken by strstr\nBasis_Set STO-3G\nMethod   CCSDT-1a  \n"
            "convergance_criteria -9\nFreeze_Core true\nuse_angstrom true\n"
            "O   0.0   0.0    0.0\nH 0   1.079252   1.474611\nH\t0 1.079252 -1.47611\n")
    p = cg.parse_incar(text, basis)  # no "#ATOMS START": the atom lines are still read
    assert p["method"] == "CCSDT-1a" and p["tol"] == pytest.approx(1e-9)
    assert p["freeze_core"] and p["nfrozen"] == 1  # the O 1s
    np.testing.assert_allclose(p["R"][1], np.array([0, 1.079252, 1.474611]) * 1.889725989, rtol=1e-15)
    for bad, code in (("Basis_Set STO-3G\nO 0 0 0\n", _abi.CCSD_ERR_INVALID_ARG),  # no Method
                      ("Method HF\n", _abi.CCSD_ERR_INVALID_ARG),  # no atoms
                      ("Method HF\n#ATOMS START\nO 0 0\n#\n", _abi.CCSD_ERR_INVALID_ARG),  # short atom line
                      ("Method HF\nNe 0 0 0\n", _abi.CCSD_ERR_INVALID_ARG)):  # element missing from the basis
        with pytest.raises(cg.CCSDError) as ei:
            cg.parse_incar(bad, basis)
        assert ei.value.code == code


def test_unbuilt_methods_are_refused_before_any_compute():
    d = np.load(GOLD / "ints_h2o_sto3g.npz")
    for m in ("UCCSDT", "CCSDT--Q"):
        with pytest.raises(cg.CCSDError) as ei:
            cg.run_incar(incar_text(d, m, -8), g94_from_fixture(d))
        assert ei.value.code == _abi.CCSD_ERR_UNSUPPORTED


def test_basis_file_keyword(tmp_path):
    """With no basis text the INCAR's Basis_File line names the Gaussian94 file."""
    d = np.load(GOLD / "ints_h2o_631g.npz")
    path = tmp_path / "water.g94"
    path.write_text(g94_from_fixture(d))
    p = cg.parse_incar(incar_text(d, "HF", -10, extra=f"Basis_File {path}"))
    np.testing.assert_allclose(p["coef"], d["coef"][:, :p["coef"].shape[1]], rtol=1e-14, atol=0)
    with pytest.raises(cg.CCSDError) as ei:
        cg.parse_incar(incar_text(d, "HF", -10))
    assert ei.value.code == _abi.CCSD_ERR_INVALID_ARG


def test_gaussian94_forms():
    """SP (and its synonym L) shells give S then P from one exponent list; Fortran
    D exponents; '!' comments and blank lines are skipped."""
    incar = "Method HF\nH 0 0 0\nLi 0 0 3.0\n"
    basis = ("! a hand-written basis\n\nH 0\nS 2 1.00\n  3.0D+00  0.5\n  0.5D0 0.6\n****\n"
             "Li 0\nS 1 1.00\n 16.0 1.0\nSP 2 1.00\n 1.5 0.3 0.2\n 0.2 0.7 0.8\n"
             "L 1 1.00\n 0.05 1.0 1.0\n****\n")
    p = cg.parse_incar(incar, basis)
    assert p["n_electrons"] == 4
    # H: 1 s; Li: s, (s, p x3) from SP, (s, p x3) from L
    np.testing.assert_array_equal(p["atom"], [0] + [1] * 9)
    np.testing.assert_array_equal(p["powers"].sum(axis=1), [0, 0, 0, 1, 1, 1, 0, 1, 1, 1])
    np.testing.assert_array_equal(p["nprim"], [2, 1, 2, 2, 2, 2, 1, 1, 1, 1])
    assert p["alpha"][0, 0] == 3.0 and p["alpha"][0, 1] == 0.5
    # an s primitive carries (2a/pi)^{3/4}, a p_x primitive (2a/pi)^{3/4} (4a)^{1/2}
    a = 1.5
    assert p["coef"][2, 0] == pytest.approx(0.3 * (2 * a / np.pi) ** 0.75, rel=1e-15)
    assert p["coef"][3, 0] == pytest.approx(0.2 * (2 * a / np.pi) ** 0.75 * np.sqrt(4 * a), rel=1e-15)


@pytest.mark.parametrize("basis,msg", [
    ("H 0\nS 2 1.00\n 3.0 0.5\n****\n", "expected an exponent"),  # '****' read as the 2nd primitive
    ("H 0\nS 2 1.00\n 3.0 0.5\n", "missing primitive lines"),
    ("H 0\nS 1 1.00\n -3.0 0.5\n****\n", "bad exponent"),
    ("H 0\nG 1 1.00\n 3.0 0.5\n****\n", "shell type"),
    ("H 0\nSP 1 1.00\n 3.0 0.5\n****\n", "coefficient"),
    ("Xx 0\nS 1 1.00\n 3.0 0.5\n****\n", "unknown element"),
])
def test_gaussian94_errors_name_the_line(basis, msg):
    with pytest.raises(cg.CCSDError) as ei:
        cg.parse_incar("Method HF\nH 0 0 0\nH 0 0 1.4\n", basis)
    assert ei.value.code == _abi.CCSD_ERR_INVALID_ARG
    assert msg in str(ei.value) and "line" in str(ei.value)
