"""Closed-shell Hartree-Fock on the GPU integrals (ccsd_rhf) against the
reference's own SCF (Hartree_Fock_Solver::get_Energy, compiled unchanged;
tests/golden/ints_*.npz) and, end to end, RHF -> CCSD against the reference's
CCSD on the same molecule (tests/golden/h2o_631g_config_tol10.npz).

Tolerances: E_HF 1e-10 (the SCF runs the reference's steps, so the fixed point
and the stopping step agree; what is left is rounding); the density
P = 2 C_occ C_occ^T and the occupied orbital energies 1e-8 (the reference stops
on the orbital-energy sum at 1e-10, so the last step moves these by about its
square root); CCSD energies 1e-9 with the reference's iteration counter."""
import json
from pathlib import Path

import numpy as np
import pytest

import ccsd_parallel_gb300 as cg
from ccsd_parallel_gb300 import _abi

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).parent / "golden"
CASES = ["h2o_sto3g", "nh3_sto3g", "h2o_631g", "h2o_ccpvdz", "o_ccpvtz"]


def _density(C, nocc):
    return 2.0 * C[:, :nocc] @ C[:, :nocc].T


@pytest.mark.parametrize("name", CASES)
def test_rhf_matches_reference(name):
    d = np.load(GOLD / f"ints_{name}.npz")
    nelec = int(d["nelec"])
    r = cg.rhf(d, nelec, tol=10.0 ** float(d["log10_tol"]))
    assert r["converged"]
    assert abs(r["e_hf"] - float(d["e_hf"])) < 1e-10
    assert abs(r["e_nuc"] - float(d["e_nuc"])) < 1e-12
    nocc = nelec // 2
    np.testing.assert_allclose(r["eps"][:nocc + 1], d["eps"][:nocc + 1], rtol=0, atol=1e-8)
    # closed-shell O empties one of the three 2p orbitals: three equivalent solutions,
    # the reference and the engine can land on different ones (same energies)
    if name != "o_ccpvtz":
        np.testing.assert_allclose(_density(r["C"], nocc), _density(d["C"], nocc), rtol=0, atol=1e-8)
    # C^T S C = 1 and the eigen-equation F C = S C eps hold for the returned orbitals
    ints = cg.ao_integrals(d, eri=False)
    S = ints["S"]
    np.testing.assert_allclose(r["C"].T @ S @ r["C"], np.eye(S.shape[0]), rtol=0, atol=1e-10)


def test_rhf_then_ccsd_matches_reference():
    """H2O 6-31G from the basis description alone: GPU integrals, GPU RHF, GPU
    CCSD; the reference's RHF + dense CCSD gave E_corr and its iteration count."""
    d = np.load(GOLD / "ints_h2o_631g.npz")
    h = np.load(GOLD / "h2o_631g_config_tol10.npz")
    scf = cg.rhf(d, 10, tol=1e-10)
    assert abs(scf["e_hf"] - float(h["e_hf"])) < 1e-10
    r = cg.solve(**cg.ccsd_inputs(scf), energy_tol=10.0 ** float(h["log10_tol"]))
    assert r["iterations"] + 1 == int(h["ref_ccsd1_iter"])
    assert abs(r["e_corr"] - float(h["ref_ccsd1_e_corr"])) < 1e-9


def test_rhf_rejects_bad_electron_counts():
    d = np.load(GOLD / "ints_h2o_sto3g.npz")
    for ne in (0, 9, 16):
        with pytest.raises(cg.CCSDError) as ei:
            cg.rhf(d, ne)
        assert ei.value.code == _abi.CCSD_ERR_INVALID_ARG


UHF = json.loads((GOLD / "reference_uhf.json").read_text())


@pytest.mark.parametrize("case", UHF, ids=[f"{c['basis_fixture'][5:-4]}_{c['n_up']}{c['n_down']}" for c in UHF])
def test_uhf_matches_reference(case):
    """The reference's UHF (get_Energy(toler, 1)) on open shells: OH doublets, H2O+
    and the H2O triplet.  Its stopping rule (the lowest orbital energy of each spin
    settles to 1e-10) leaves the energy good to about 1e-10, and it starts from
    random densities; energies within 1e-9, for two seeds of the engine's start."""
    d = np.load(GOLD / case["basis_fixture"])
    for seed in (0, 7):
        r = cg.uhf(d, case["n_up"], case["n_down"], tol=10.0 ** case["log10_tol"], seed=seed)
        assert r["converged"]
        assert abs(r["e_uhf"] - case["e_uhf"]) < 1e-9
