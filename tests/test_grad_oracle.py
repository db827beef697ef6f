"""CPU: the host FP64 Lambda/gradient reference (oracle.ccsd_grad, torch
autograd over the closed-shell residual) against central finite differences
of the converged CCSD energy of the oracle (oracle.ccsd_rhf)."""
import itertools

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import synthetic as syn
from oracle.ccsd_grad import lambda_grad
from oracle.ccsd_rhf import RHFCCSD


def read_positions(o, v, rng, k, blocks=None):
    """Integral entries the closed-shell equations read (the other entries of
    the dense tensor have derivative 0)."""
    n = o + v
    allb = {"ovov": ((0, o), (o, n), (0, o), (o, n)), "oovv": ((0, o), (0, o), (o, n), (o, n)),
            "ovoo": ((0, o), (o, n), (0, o), (0, o)), "oooo": ((0, o), (0, o), (0, o), (0, o)),
            "ovvv": ((0, o), (o, n), (o, n), (o, n)), "vvvv": ((o, n), (o, n), (o, n), (o, n))}
    names = blocks or sorted(allb)
    out = []
    for _ in range(k):
        b = allb[names[rng.integers(0, len(names))]]
        out.append(tuple(int(rng.integers(a, c)) for a, c in b))
    return out


def orbit(idx):
    """The 8 index orders of (pq|rs) that real orbitals make equal."""
    p, q, r, s = idx
    return sorted({(p, q, r, s), (q, p, r, s), (p, q, s, r), (q, p, s, r),
                   (r, s, p, q), (s, r, p, q), (r, s, q, p), (s, r, q, p)})


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
    # The oracle reads the ladder's inputs as given, the restatement (like the
    # engine) symmetrised; their per-element derivatives differ but agree on
    # symmetric perturbations: the 8-permutation orbit of an entry.
    for idx in read_positions(o, v, rng, 10):
        orb = orbit(idx)
        gp, gm = eri.copy(), eri.copy()
        for e in orb:
            gp[e] += h
            gm[e] -= h
        fd = (E(fock, gp) - E(fock, gm)) / (2 * h)
        assert abs(fd - sum(G["d_eri"][e] for e in orb)) < 1e-9, idx
    for idx in [(0, 0), (1, 2), (o, o + 1), (0, o + 2), (o + 1, 0)]:
        fp, fm = fock.copy(), fock.copy()
        fp[idx] += h
        fm[idx] -= h
        assert abs((E(fp, eri) - E(fm, eri)) / (2 * h) - G["d_fock"][idx]) < 1e-9


def test_orbit_sums_do_not_depend_on_the_ladder_convention():
    """Symmetrising the ladder's inputs changes per-element derivatives (through
    the antisymmetric part of Lambda2) but not their sums over the permutation
    orbit, nor dE/dfock."""
    import oracle.ccsd_grad as cgm
    o, v = 2, 5
    eps = syn.orbital_energies(o, v, 6)
    eri = syn.eri_from_df(syn.df_factors(o + v, 12, 6, sigma=0.3))
    fock = np.diag(eps)
    r = RHFCCSD(fock, o, eri=eri).run(toler=1e-13)
    G = lambda_grad(fock, eri, o, r["t1"], r["t2"], tol=1e-13)
    orig = cgm.numerators

    def plain(t1, t2, f, g, o_):  # the same equations with the ladder read as given
        R1, R2, D1, D2 = orig(t1, t2, f, g, o_)
        vvvv = g[o_:, o_:, o_:, o_:]
        tau = t2 + torch.einsum("ia,jb->ijab", t1, t1)
        R2 = (R2 - torch.einsum("acbd,ijcd->ijab", 0.5 * (vvvv + vvvv.permute(2, 3, 0, 1)),
                                0.5 * (tau + tau.permute(1, 0, 3, 2)))
              + torch.einsum("acbd,ijcd->ijab", vvvv, tau))
        return R1, R2, D1, D2

    cgm.numerators = plain
    try:
        Gp = lambda_grad(fock, eri, o, r["t1"], r["t2"], tol=1e-13)
    finally:
        cgm.numerators = orig
    np.testing.assert_allclose(G["d_fock"], Gp["d_fock"], rtol=0, atol=1e-12)
    n = o + v
    for idx in itertools.product(range(n), repeat=4):
        orb = orbit(idx)
        assert abs(sum(G["d_eri"][e] for e in orb) - sum(Gp["d_eri"][e] for e in orb)) < 1e-12
