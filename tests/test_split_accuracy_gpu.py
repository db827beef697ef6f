"""Accuracy of the split-precision tensor-core path at the benchmark shapes.

The target: |dE_corr| <= 1e-8 Eh against FP64, with max|dT2| stated.
* o=10, v=90, naux=300, seed 2024: every per-update energy of split2/3/4 against
  the oracle's (tests/golden/synthetic_oracle.json), and T2 against the FP64
  GPU path (itself equal to the oracle to 1e-12 in test_parity_gpu.py);
* o=24, v=300, naux=900, seed 2024 (the benchmark workload, ~150 GB of device
  memory per solve): 3 DIIS(6) updates of split3 against the FP64 path.
"""
import json
from pathlib import Path

import numpy as np
import pytest

import ccsd_parallel_gb300 as cg

pytestmark = pytest.mark.gpu

GOLDEN = json.loads((Path(__file__).parent / "golden" / "synthetic_oracle.json").read_text())
C2 = GOLDEN["syn_o10_v90_q300_s2024_sig0.05"]


@pytest.fixture(scope="module")
def c2_fp64():
    fock, b = cg.make_synthetic(C2["nocc"], C2["nvir"], C2["naux"], C2["seed"])
    r = cg.solve(fock, C2["nocc"], df=b, fixed_iterations=C2["iter"] - 1)
    np.testing.assert_allclose(r["energies"], C2["energies"], rtol=0, atol=1e-12)
    return fock, b, r


@pytest.mark.parametrize("precision,t2_bound", [("split2", 1e-7), ("split3", 1e-10), ("split4", 1e-10)])
def test_split_c2_energies_and_amplitudes(c2_fp64, precision, t2_bound):
    fock, b, r64 = c2_fp64
    r = cg.solve(fock, C2["nocc"], df=b, fixed_iterations=C2["iter"] - 1, precision=precision)
    de = np.abs(r["energies"] - np.asarray(C2["energies"])).max()
    dt2 = np.abs(r["t2"] - r64["t2"]).max()
    print(f"C2 {precision}: max|dE| vs oracle {de:.2e} Eh, max|dT2| vs FP64 {dt2:.2e}")
    assert de <= 1e-8
    assert dt2 <= t2_bound


def test_split3_benchmark_workload_against_fp64():
    o, v, q = 24, 300, 900
    fock, b = cg.make_synthetic(o, v, q, 2024)
    kw = dict(fixed_iterations=3, diis_size=6, diis_start=2)
    rs = cg.solve(fock, o, df=b, precision="split3", **kw)
    r64 = cg.solve(fock, o, df=b, precision="fp64", **kw)
    de = np.abs(rs["energies"] - r64["energies"]).max()
    dt2 = np.abs(rs["t2"] - r64["t2"]).max()
    print(f"C5 split3: max|dE| vs FP64 {de:.2e} Eh, max|dT2| {dt2:.2e} (|T2|max {np.abs(r64['t2']).max():.2e})")
    assert de <= 1e-8
    assert dt2 <= 1e-8
