"""The INCAR front end end to end (ccsd_incar_run = the reference's
Initializer::Go on the engine): an INCAR and a Gaussian94 basis give the
energies the reference printed for H2O 6-31G (tests/golden/ints_h2o_631g.npz,
h2o_631g_config_tol10.npz, reference_ccsdt1a.json): HF to 1e-10, CCSD and
CCSDT-1a to 1e-9 with the reference's iteration counter."""
import json
from pathlib import Path

import numpy as np
import pytest

import ccsd_parallel_gb300 as cg
from incar_util import g94_from_fixture, incar_text

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).parent / "golden"


def _inputs():
    return np.load(GOLD / "ints_h2o_631g.npz"), np.load(GOLD / "h2o_631g_config_tol10.npz")


def test_incar_hf():
    d, _ = _inputs()
    r = cg.run_incar(incar_text(d, "HF", -10), g94_from_fixture(d))
    assert r["method"] == -1 and r["cc_iter"] == 0
    assert abs(r["energy"] - float(d["e_hf"])) < 1e-10


def test_incar_ccsd_and_units():
    d, h = _inputs()
    basis = g94_from_fixture(d)
    # "CCSD" runs the memory-optimised class in the reference (initializer.cpp:191-195)
    r = cg.run_incar(incar_text(d, "CCSD", -10), basis)
    assert r["cc_iter"] == int(h["ref_iter"])
    assert abs(r["energy"] - float(h["ref_e_total"])) < 1e-9
    # "CCSD1" runs its dense spin-orbital CCSD (initializer.cpp:98-103)
    r1 = cg.run_incar(incar_text(d, "CCSD1", -10), basis)
    assert r1["cc_iter"] == int(h["ref_ccsd1_iter"])
    assert abs(r1["energy"] - (float(h["e_hf"]) + float(h["ref_ccsd1_e_corr"]))) < 1e-9
    # the same molecule in angstrom
    ra = cg.run_incar(incar_text(d, "CCSD", -10, angstrom=True), basis)
    assert abs(ra["energy"] - r["energy"]) < 1e-9


def test_incar_ccsdt1a():
    d, h = _inputs()
    ref = json.loads((GOLD / "reference_ccsdt1a.json").read_text())["h2o"]["h2o_631g_config_tol10.npz"]
    r = cg.run_incar(incar_text(d, "CCSDT-1a", -10), g94_from_fixture(d))
    assert r["cc_iter"] == ref["iter"]
    assert abs(r["e_corr"] - ref["e_corr"]) < 1e-9
    assert abs(r["energy"] - (float(h["e_hf"]) + ref["e_corr"])) < 1e-9


def test_incar_uhf_triplet():
    """Method UHF with 10 electrons: Go runs the singlet, then returns the triplet
    (6 up, 4 down); the reference's triplet H2O STO-3G energy."""
    d = np.load(GOLD / "ints_h2o_sto3g.npz")
    ref = [c for c in json.loads((GOLD / "reference_uhf.json").read_text())
           if c["basis_fixture"] == "ints_h2o_sto3g.npz" and c["n_up"] == 6][0]
    r = cg.run_incar(incar_text(d, "UHF", -10), g94_from_fixture(d))
    assert r["method"] == -2
    assert abs(r["energy"] - ref["e_uhf"]) < 1e-9
