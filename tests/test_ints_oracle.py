"""The integral oracle (oracle/gto_ints.py) pinned to the reference's own
integrals (tests/golden/ints_*.npz, written by make_ints_golden.py from the
reference's Hartree_Integrals / Hartree_Fock_Solver compiled unchanged):
S, <mu|nabla^2|nu>, sum_C Z_C <mu|1/r_C|nu> and E_nuc whole, the ERIs on a sample.
Tolerance 1e-13 absolute (5e-14 measured at worst)."""
from pathlib import Path

import numpy as np
import pytest

from oracle.gto_ints import Basis, Integrals, boys

GOLD = Path(__file__).parent / "golden"
CASES = ["h2o_sto3g", "nh3_sto3g", "h2o_631g", "h2o_ccpvdz", "o_ccpvtz"]


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference_integrals(name):
    d = np.load(GOLD / f"ints_{name}.npz")
    I = Integrals(Basis.from_dict(d))
    np.testing.assert_allclose(I.overlap(), d["S"], rtol=0, atol=1e-13)
    np.testing.assert_allclose(I.laplacian(), d["lap"], rtol=0, atol=1e-13)
    np.testing.assert_allclose(I.nuclear(), d["nuc"], rtol=0, atol=1e-12)
    assert abs(I.nuclear_repulsion() - float(d["e_nuc"])) < 1e-12
    if "eri" in d:
        n = d["S"].shape[0]
        rng = np.random.default_rng(1)
        idx = rng.integers(0, n, size=(40, 4))
        vals = d["eri"][tuple(idx.T)]
    else:
        idx, vals = d["eri_idx"][::75], d["eri_val"][::75]
    for q, v in zip(idx, vals):
        assert abs(I.eri(*map(int, q)) - v) < 1e-13


def test_boys_function_limits():
    """F_n(0) = 1/(2n+1).  At x = 50 the reference's asymptotic F_30
    (hartree_integrals.cpp:656-666) jumps by 1.2e-3 (relative) from its series,
    which is right there (F_0(50) = sqrt(pi/50)/2 to e^-50); the accurate form is
    continuous.  Above x = 1.1e5 the reference's x^61 overflows and every F_n is 0."""
    F = boys(12, 0.0)
    np.testing.assert_allclose(F, 1.0 / (2 * np.arange(13) + 1), rtol=1e-15)
    lo, hi = boys(8, 50.0), boys(8, 50.0 + 1e-9)
    assert abs(lo[0] - 0.5 * np.sqrt(np.pi / 50.0)) < 1e-16
    np.testing.assert_allclose(hi / lo - 1.0, 1.2137e-3, rtol=1e-3)
    np.testing.assert_allclose(boys(8, 50.0 + 1e-9, as_written=False), lo, rtol=1e-8)
    assert not boys(4, 2e5).any() and boys(4, 2e5, as_written=False)[0] > 0
