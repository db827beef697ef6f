"""CPU: the host FP64 Lambda/gradient reference (oracle.ccsd_grad, torch
autograd over the closed-shell residual) against central finite differences
of the converged CCSD energy."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import synthetic as syn
from oracle.ccsd_grad import lambda_grad
from oracle.ccsd_rhf import RHFCCSD


def read_positions(o, v, rng, k):
    """Integral entries the closed-shell equations read (the other entries of
    the dense tensor have derivative 0)."""
    n = o + v
    blocks = [((0, o), (o, n), (0, o), (o, n)), ((0, o), (0, o), (o, n), (o, n)), ((0, o), (o, n), (0, o), (0, o)),
              ((0, o), (0, o), (0, o), (0, o)), ((0, o), (o, n), (o, n), (o, n)), ((o, n), (o, n), (o, n), (o, n))]
    return [tuple(int(rng.integers(a, b)) for a, b in blocks[rng.integers(0, 6)]) for _ in range(k)]


def test_lambda_reference_matches_finite_differences():
    o, v = 3, 6
    eps = syn.orbital_energies(o, v, 4)
    eri = syn.eri_from_df(syn.df_factors(o + v, 15, 4, sigma=0.3))
    rng = np.random.default_rng(1)
    x = 0.01 * rng.standard_normal((o + v, o + v))
    fock = np.diag(eps) + x + x.T

    def E(fk, g):
        return RHFCCSD(fk, o, eri=g).run(toler=1e-13)["e_corr"]

    r = RHFCCSD(fock, o, eri=eri).run(toler=1e-13)
    G = lambda_grad(fock, eri, o, r["t1"], r["t2"])
    h = 1e-5
    for idx in read_positions(o, v, rng, 8):
        gp, gm = eri.copy(), eri.copy()
        gp[idx] += h
        gm[idx] -= h
        assert abs((E(fock, gp) - E(fock, gm)) / (2 * h) - G["d_eri"][idx]) < 1e-9
    for idx in [(0, 0), (1, 2), (o, o + 1), (0, o + 2), (o + 1, 0)]:
        fp, fm = fock.copy(), fock.copy()
        fp[idx] += h
        fm[idx] -= h
        assert abs((E(fp, eri) - E(fm, eri)) / (2 * h) - G["d_fock"][idx]) < 1e-9
