"""The SCF oracle (oracle/scf.py) pinned to the reference's own Hartree-Fock runs
on the reference's own integrals (tests/golden/ints_*.npz, reference_uhf.json):
RHF energies, densities and orbital energies to 1e-12 (the steps are the same;
what is left is rounding), UHF energies to 1e-9 from two seeds (the reference
starts from random densities and stops on the lowest orbital energies)."""
import json
from pathlib import Path

import numpy as np
import pytest

from oracle.scf import rhf, uhf

GOLD = Path(__file__).parent / "golden"


def _ints(d):
    return d["S"], -0.5 * d["lap"] - d["nuc"], d["eri"], float(d["e_nuc"])


@pytest.mark.parametrize("name", ["h2o_sto3g", "nh3_sto3g", "h2o_631g"])
def test_rhf_oracle_matches_reference(name):
    d = np.load(GOLD / f"ints_{name}.npz")
    S, h, G, en = _ints(d)
    r = rhf(S, h, G, en, int(d["nelec"]), tol=10.0 ** float(d["log10_tol"]))
    nocc = int(d["nelec"]) // 2
    assert abs(r["e_hf"] - float(d["e_hf"])) < 1e-12
    np.testing.assert_allclose(r["eps"], d["eps"], rtol=0, atol=1e-12)
    P, Pr = (2 * C[:, :nocc] @ C[:, :nocc].T for C in (r["C"], d["C"]))
    np.testing.assert_allclose(P, Pr, rtol=0, atol=1e-12)


@pytest.mark.parametrize("case", json.loads((GOLD / "reference_uhf.json").read_text()),
                         ids=lambda c: f"{c['basis_fixture'][5:-4]}_{c['n_up']}{c['n_down']}")
def test_uhf_oracle_matches_reference(case):
    d = np.load(GOLD / case["basis_fixture"])
    S, h, G, en = _ints(d)
    for seed in (0, 1):
        r = uhf(S, h, G, en, case["n_up"], case["n_down"], tol=10.0 ** case["log10_tol"], seed=seed)
        assert abs(r["e_uhf"] - case["e_uhf"]) < 1e-9
